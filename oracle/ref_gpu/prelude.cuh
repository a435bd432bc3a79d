/*
 * prelude.cuh -- included ahead of the reference's main.h and kernel
 * section (main.cu from InitQPSO up to main()) when they are compiled for
 * sm_103a into oracle/_ref/ by oracle/build.py.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing of the reference is copied into this
 * repository: the recipe reads the sources where they lie and writes only
 * the cubins.  Two shims make the 2016 code compile for sm_103a:
 *   - __ballot (removed for sm_70 and later) becomes __ballot_sync over the
 *     lanes active at the call, which is what __ballot(1) returned on the
 *     GPUs the reference was written for (main.cu:722);
 *   - -DdeviceOverlap=asyncEngineCount on the command line, because CUDA 13
 *     removed the cudaDeviceProp field that main.h:1178 reads in a host
 *     function the kernels never call.
 * The OpenCV and assimp names main.h mentions come from the
 * declaration-only stand-ins in oracle/ref_pin/stubs.
 */
#pragma once
#include <cstdint>
#include <cstdio>
#include <iostream>
#include <vector>
#include <cuda_runtime.h>
#include <vector_types.h>
#define __ballot(pred) __ballot_sync(__activemask(), (pred))

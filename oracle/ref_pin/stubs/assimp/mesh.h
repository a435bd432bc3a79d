#include "cimport.h"

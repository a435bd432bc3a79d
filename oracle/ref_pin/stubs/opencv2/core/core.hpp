/* Declaration-only stand-in for the OpenCV type the reference's main.h uses
 * in two global declarations. */
#ifndef QPSO_PIN_CV_STUB_H
#define QPSO_PIN_CV_STUB_H
namespace cv { struct Mat { int rows = 0, cols = 0; }; }
#endif

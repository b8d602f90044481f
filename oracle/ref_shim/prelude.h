// TEST INFRASTRUCTURE ONLY -- included before every reference source compiled
// by oracle/build_ref.py.
// * The reference's helper_cuda.h (a CUDA 8 sample header) names cuFFT and
//   device-property fields that CUDA 13 removed.  Nothing on the compiled CPU
//   path calls into CUDA, so its guard is defined to skip it, and the one
//   macro the reference's memory manager uses from it (in a CUDA template
//   that the CPU path never instantiates) is given a plain definition.
// * MSVC's standard headers (and OpenCV's, which the reference includes
//   everywhere) make std::logic_error, std::cout and std::vector visible
//   without their own headers; GCC's do not.
#ifndef TWREF_PRELUDE_H
#define TWREF_PRELUDE_H
#define HELPER_CUDA_H
#define checkCudaErrors(val) (val)
#include <stdexcept>
#include <iostream>
#include <vector>
#include <cmath>
#include <algorithm>
#include <limits>
#include <string>
#endif

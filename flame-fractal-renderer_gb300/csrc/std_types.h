// Fixed-width integer types for the headers that three compilers read: the
// host compiler, nvcc (the ahead-of-time kernel objects) and NVRTC (the
// per-flame kernels compiled at run time, jit.cpp), which provides no C++
// standard library headers.  The NVRTC definitions are the LP64 ones glibc
// gives the other two, so templates see the same types in all three.
#pragma once

#ifdef __CUDACC_RTC__
typedef signed char int8_t;
typedef unsigned char uint8_t;
typedef short int16_t;
typedef unsigned short uint16_t;
typedef int int32_t;
typedef unsigned int uint32_t;
typedef long int64_t;
typedef unsigned long uint64_t;
#else
#include <cstddef>
#include <cstdint>
#include <cstring>
#endif

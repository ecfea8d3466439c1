// Stand-in CUDA runtime names used by lib/include/optixUtils.hpp (no GPU here).
#pragma once
#include <cstddef>
typedef int cudaError_t;
static const cudaError_t cudaSuccess = 0;
inline const char* cudaGetErrorString(cudaError_t) { return "no error"; }
inline cudaError_t cudaFree(void*) { return cudaSuccess; }
struct uint3 { unsigned int x, y, z; };
#ifndef __align__
#define __align__(n) __attribute__((aligned(n)))
#endif

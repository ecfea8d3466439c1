// Stand-in OptiX names used by lib/include/optixUtils.hpp and intersections.hpp.
// The context is inert; visibility comes from the oracle (ref_shim.cpp).
#pragma once
#include "cuda_runtime.h"
typedef int OptixResult;
static const OptixResult OPTIX_SUCCESS = 0;
typedef struct OptixDeviceContext_t* OptixDeviceContext;
typedef unsigned long long OptixTraversableHandle;
struct OptixDeviceContextOptions { void* logCallbackFunction; int logCallbackLevel; };
#define OPTIX_SBT_RECORD_ALIGNMENT 16
#define OPTIX_SBT_RECORD_HEADER_SIZE 32
typedef struct CUctx_st* CUcontext;
typedef int CUresult;
static const CUresult CUDA_SUCCESS = 0;
inline CUresult cuCtxGetCurrent(CUcontext* c) { *c = reinterpret_cast<CUcontext>(0x1); return CUDA_SUCCESS; }
inline OptixResult optixInit() { return OPTIX_SUCCESS; }
inline OptixResult optixDeviceContextCreate(CUcontext, const OptixDeviceContextOptions*, OptixDeviceContext* c) {
  *c = reinterpret_cast<OptixDeviceContext>(0x1);
  return OPTIX_SUCCESS;
}
inline OptixResult optixDeviceContextDestroy(OptixDeviceContext) { return OPTIX_SUCCESS; }

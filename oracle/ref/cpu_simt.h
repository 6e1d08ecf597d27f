// Force-included shim that lets the reference's own CUDA kernel sources
// (include/OpenSteer/CUDA/*Kernel.cu of PsychoLogicAu/GPUSteer) compile with
// g++ and run on the CPU, so that their outputs can pin the oracle.
//
// TEST INFRASTRUCTURE ONLY: used by oracle/ref/gsref.cpp to generate the
// golden fixtures under tests/golden/.  Nothing here ships.
//
// What it provides:
//  * the CUDA function/variable qualifiers; __shared__ becomes thread_local,
//    so a block's emulated threads (fibers on one OS thread) share it,
//  * threadIdx/blockIdx/blockDim/gridDim and a __syncthreads() that is a real
//    barrier over the block's fibers (see gsref_simt.cpp),
//  * the legacy texture-reference API (texture<>, cudaBindTexture,
//    tex1Dfetch, tex3D with normalised point sampling and clamp addressing
//    as the CUDA Programming Guide's texture-fetching appendix specifies),
//  * stand-ins for the host headers the kernel files reach through their
//    include chains (their include guards are pre-defined below so that the
//    Windows / cutil / host-class headers are not pulled in).
#ifndef GSREF_CPU_SIMT_H
#define GSREF_CPU_SIMT_H

#define __global__
#define __device__
#define __host__
#define __shared__ thread_local
#define __constant__

#include <vector_types.h>
#include <vector_functions.h>
#include <driver_types.h>
#include <texture_types.h>

#include <cfloat>
#include <climits>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <iostream>

typedef unsigned int uint;

// CUDA device code sees binary32 overloads of the math functions in the global
// namespace, so the kernels' sqrt(float) is a binary32 square root and
// `maxLength / sqrt(lenSq)` (VectorUtils.cuh:188) is a binary32 division.
// Host g++ would otherwise pick ::sqrt(double) and divide in binary64.
inline float sqrt(float x) { return std::sqrt(x); }
inline float fabs(float x) { return std::fabs(x); }

// ---- launch geometry and barrier --------------------------------------------
extern uint3 gsref_threadIdx, gsref_blockIdx;
extern dim3 gsref_blockDim, gsref_gridDim;
void gsref_syncthreads();
#define threadIdx gsref_threadIdx
#define blockIdx gsref_blockIdx
#define blockDim gsref_blockDim
#define gridDim gsref_gridDim
#define __syncthreads() gsref_syncthreads()

// ---- cutil ------------------------------------------------------------------
#define CUDA_SAFE_CALL(call) (call)
#define cutilCheckMsg(msg) ((void)0)

// ---- legacy texture references -------------------------------------------------
struct gsref_array3d {
    const unsigned* data;
    unsigned w, h, d;
};

template <class T, int Dim = cudaTextureType1D,
          enum cudaTextureReadMode Mode = cudaReadModeElementType>
struct texture {
    int normalized = 0;
    enum cudaTextureFilterMode filterMode = cudaFilterModePoint;
    enum cudaTextureAddressMode addressMode[3] = {cudaAddressModeClamp, cudaAddressModeClamp,
                                                  cudaAddressModeClamp};
    const T* data = nullptr;
    size_t count = 0;
    const gsref_array3d* array = nullptr;
};

template <class T> inline cudaChannelFormatDesc cudaCreateChannelDesc() {
    return cudaChannelFormatDesc{};
}

template <class T, int D, enum cudaTextureReadMode M>
inline cudaError_t cudaBindTexture(size_t*, texture<T, D, M>& t, const void* p,
                                   const cudaChannelFormatDesc&, size_t bytes) {
    t.data = static_cast<const T*>(p);
    t.count = bytes / sizeof(T);
    return cudaSuccess;
}
template <class T, int D, enum cudaTextureReadMode M>
inline cudaError_t cudaBindTextureToArray(texture<T, D, M>& t, const cudaArray* a,
                                          const cudaChannelFormatDesc&) {
    t.array = reinterpret_cast<const gsref_array3d*>(a);
    return cudaSuccess;
}
template <class T, int D, enum cudaTextureReadMode M>
inline cudaError_t cudaUnbindTexture(texture<T, D, M>& t) {
    t.data = nullptr;
    t.count = 0;
    t.array = nullptr;
    return cudaSuccess;
}

// Linear-memory fetch; out-of-range fetches return zero.
template <class T, int D, enum cudaTextureReadMode M>
inline T tex1Dfetch(const texture<T, D, M>& t, int i) {
    if (i < 0 || size_t(i) >= t.count) return T{};
    return t.data[i];
}

// Normalised coordinates, nearest-point sampling, clamp addressing:
// texel i = clamp(floor(x * N), 0, N - 1) per axis.
inline unsigned gsref_texel(float x, unsigned n) {
    const float f = std::floor(x * float(n));
    if (!(f >= 0.f)) return 0u;
    if (f >= float(n)) return n - 1;
    return unsigned(f);
}
template <class T, int D, enum cudaTextureReadMode M>
inline T tex3D(const texture<T, D, M>& t, float x, float y, float z) {
    const gsref_array3d* a = t.array;
    const unsigned tx = gsref_texel(x, a->w), ty = gsref_texel(y, a->h), tz = gsref_texel(z, a->d);
    return T(a->data[tx + ty * a->w + tz * a->w * a->h]);
}

// ---- headers cut out of the include chains -------------------------------------
#define CUDA_GLOBALS_H                         /* CUDA/CUDAGlobals.cuh (windows.h, cutil) */
#define OPENSTEER_AGENTGROUPDATA_CUH           /* AgentGroupData.cuh (dev_vector, host data) */
#define OPENSTEER_KNNBINNINGV2_CUH             /* host wrapper classes */
#define OPENSTEER_STEERFORSEPARATIONCUDA_H
#define OPENSTEER_STEERFORCOHESIONCUDA_H
#define OPENSTEER_STEERFORALIGNMENTCUDE_CUH
#define OPENSTEER_ANTIPENETRATIONAGENTSCUDA_CUH
#define UPDATECUDA_H
#define OPENSTEER_STEERTOFOLLOWPATHCUDA_CUH     /* host wrapper class (AbstractCUDAKernel) */
#define KNN_THREADSPERBLOCK 128                /* KNNBinDataV2.cuh:13 */

#include <OpenSteer/CUDA/CUDAUtils.cuh>          /* OpenSteer::swap */
#include <OpenSteer/CUDA/KNNBinDataGlobals.cuh>  /* bin_cell */
#include <OpenSteer/VectorUtils.cuh>

// AgentGroupData.cuh's velocity(): the agent's direction scaled by its speed.
static inline float3 velocity(size_t const i, float3 const* dir, float const* speed) {
    return float3_scalar_multiply(dir[i], speed[i]);
}

#include <OpenSteer/CUDA/CUDAKernelGlobals.cuh>
#include <OpenSteer/CUDA/FlockingCommon.cuh>

// Storage behind `extern __shared__` (dynamic shared memory) declarations;
// placed inside each namespace that wraps a kernel source file.
#define GSREF_DYNAMIC_SHARED                                  \
    static thread_local unsigned int shKNNIndices[1 << 15];   \
    static thread_local float shKNNDistances[1 << 15];        \
    static thread_local unsigned int shKNLIndices[1 << 14];   \
    static thread_local unsigned int shNeighboringCells[1 << 14];

#endif

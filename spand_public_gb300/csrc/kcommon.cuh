// Definitions shared by the CUDA translation units: device work-list records, the
// device context of the factorization, error checking and warp/block reductions.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "device.h"

namespace spand {

#define SPAND_CUDA(call)                                                                        \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess)                                                                  \
            throw DeviceError{SPAND_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)}; \
    } while (0)

// ------------------------------------------------------------------------------------
// Device work-list records
// ------------------------------------------------------------------------------------
struct DBlock {
    long long off;
    int ld, rowc, colc, flag;
};
struct DTrsm {
    int block, lblock, cluster, side;
};
struct DTile {
    int item, tile_i, tile_j;
};
struct DTarget {
    int target, syrk, first, count;
};
struct DUpd {
    int b1, t1, b2, t2, s;
};
struct DAsn {
    int block, nbr, transposed;
};
struct DSpars {
    int cluster, first, count, cap_cols;
    long long ws_off, col_off, v_off, tau_off;
};
struct DMerge {
    int src, dst, nold, sold;
};
struct DGemmOp {
    int self, nbr, block, kind;
};
struct DGroup {
    int key, first, count;
};
struct DOrtho {
    int cluster;
    long long v_off, tau_off;
};

// Status word: first failing cluster + 1 for a non-SPD pivot.
struct DStatus {
    int not_spd;
    int overflow;  // a sparsification matrix outgrew its wave's shared-memory QRCP launch
};

template <typename T>
struct Ctx {
    T* arena;
    const DBlock* blk;
    int* csize;
    int* rows0;
    const int* cap;
    DStatus* status;
};

template <typename T>
__device__ __forceinline__ T* bptr(const Ctx<T>& c, int b) {
    return c.arena + c.blk[b].off;
}

template <typename T>
__device__ __forceinline__ T dsqrt(T x) {
    return sqrt(x);
}

// 1 / sqrt(x): the hardware reciprocal square root in FP32 (a few ulp), correctly rounded
// sqrt and division in FP64
__device__ __forceinline__ float rsqrt_t(float x) { return rsqrtf(x); }
__device__ __forceinline__ double rsqrt_t(double x) { return 1.0 / sqrt(x); }

// four consecutive elements from shared memory, p aligned to four elements (16-byte loads)
__device__ __forceinline__ void lds4(const float* p, float (&x)[4]) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    x[0] = v.x;
    x[1] = v.y;
    x[2] = v.z;
    x[3] = v.w;
}
__device__ __forceinline__ void lds4(const double* p, double (&x)[4]) {
    const double2 v0 = *reinterpret_cast<const double2*>(p), v1 = *reinterpret_cast<const double2*>(p + 2);
    x[0] = v0.x;
    x[1] = v0.y;
    x[2] = v1.x;
    x[3] = v1.y;
}

// ------------------------------------------------------------------------------------
// Block reductions (fixed order, deterministic)
// ------------------------------------------------------------------------------------
template <typename T>
__device__ T block_sum(T v, T* red) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    T s = 0;
    if (threadIdx.x == 0) {
        for (int i = 0; i < nw; i++) s += red[i];
        red[32] = s;
    }
    __syncthreads();
    s = red[32];
    return s;
}

// Programmatic dependent launch (the solve sweep's kernels): wait until the previous
// kernel of the stream has finished and its writes are visible -- a no-op for a kernel
// launched without the attribute -- then let the next kernel's CTAs be scheduled while
// this one runs (they wait in their own griddepcontrol.wait).  Called first, before any
// read of data an earlier kernel wrote.
__device__ __forceinline__ void pdl_wait_and_release() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename T>
__device__ T warp_sum(T v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Relative window inside which partial column norms count as tied (same rule as the
// oracle's restated dgeqp3).
template <typename T>
__device__ __forceinline__ T qrcp_tie() {
    return sizeof(T) == 8 ? T(1e-7) : T(1e-4);
}

}  // namespace spand

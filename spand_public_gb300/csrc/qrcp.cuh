// QRCP of the sparsification matrices (rank-revealing Householder QR with column
// pivoting, resident in the shared memory of a thread-block cluster): what the device
// driver needs to configure and launch it.  The kernel lives in qrcp.cu.
#pragma once

#include "kcommon.cuh"

namespace spand {

constexpr int QC_THREADS = 256;

// Shared memory of one CTA holding a rows x ceil(cols/cs) column slab: the slab (ld =
// rows | 1), the reflector, two partial-norm arrays, the replicated permutation and the
// slab's column positions.
__host__ __device__ inline long long qc_need(int rows, int cols, int cs, int elem) {
    const long long cpc = (cols + cs - 1) / cs;
    return ((long long)(rows | 1) * cpc + rows + 2 * cpc) * elem + ((long long)cols + cpc) * 4;
}

// Shared memory of one CTA of the global-slab variant: the reflector, the two norm
// arrays, the replicated permutation and the slab's column positions.
__host__ __device__ inline long long qc_small_need(int rows, int cols, int cs, int elem) {
    const long long cpc = (cols + cs - 1) / cs;
    return ((long long)rows + 2 * cpc) * elem + ((long long)cols + cpc) * 4;
}

// Preservation (src/tree.cpp:1371-1373): before the QRCP, Asn <- (I - Q1 Q1^T) Asn with
// Q1 the orthonormal basis at the item's v_off in q (ld = the cluster's capacity) and
// rank1[cluster] its column count; rank1 >= rows: nothing to factor (rank 0).  q ==
// nullptr: plain QRCP.
template <typename T>
struct QcProj {
    const T* q;
    const int* rank1;
};

// (ctx, items, pieces, ws, gslab, jpvt, ipvt, tau, rank, colcount, fallback, tol,
//  dynamic shared bytes, probe, projection)
template <typename T>
using QcKernel = void (*)(Ctx<T>, const DSpars*, const DAsn*, T*, T*, int*, int*, T*, int*, int*, int*, double,
                          int, unsigned long long*, QcProj<T>);

// column slabs in the cluster's shared memory
template <typename T>
QcKernel<T> qrcp_smem_kernel_ptr();
// column slabs in global memory, for the matrices the shared-memory launch flagged
template <typename T>
QcKernel<T> qrcp_gslab_kernel_ptr();

}  // namespace spand

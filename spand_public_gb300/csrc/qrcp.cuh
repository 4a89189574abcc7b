// QRCP of the sparsification matrices (rank-revealing Householder QR with column
// pivoting, resident in the shared memory of a thread-block cluster): what the device
// driver needs to configure and launch it.  The kernel lives in qrcp.cu.
#pragma once

#include "kcommon.cuh"

namespace spand {

constexpr int QC_THREADS = 256;
// the wide instantiation of the shared-memory QRCP (one CTA per SM, 16 warps per slab)
constexpr int QC_WIDE_THREADS = 512;

// Leading dimension of a column slab in shared memory: rows | 1 (odd: the scalar update's
// column groups fall on distinct banks) or rows rounded up to whole 16-byte vectors (the
// vectorised update); the larger of the two is reserved.
__host__ __device__ inline int qc_ld_bound(int rows, int elem) {
    const int vw = 16 / elem;
    return ((rows | 1) + vw - 1) / vw * vw;
}

// Shared memory of one CTA holding a rows x ceil(cols/cs) column slab: the slab, the
// reflector (one leading dimension each), two partial-norm arrays, the replicated
// permutation and the slab's column positions.
__host__ __device__ inline long long qc_need(int rows, int cols, int cs, int elem) {
    const long long cpc = (cols + cs - 1) / cs;
    const long long ld = qc_ld_bound(rows, elem);
    return (ld * cpc + ld + 2 * cpc) * elem + ((long long)cols + cpc) * 4;
}

// Shared memory of one CTA of the global-slab variant: the reflector, the two norm
// arrays, the replicated permutation and the slab's column positions.
__host__ __device__ inline long long qc_small_need(int rows, int cols, int cs, int elem) {
    const long long cpc = (cols + cs - 1) / cs;
    return ((long long)rows + 2 * cpc) * elem + ((long long)cols + cpc) * 4;
}

// Panel width of the blocked QRCP (qrcp_blocked.cu): pivot steps between two
// applications of the accumulated reflectors to the trailing columns.
constexpr int QB_NB = 16;

// Shared memory of one CTA of the blocked QRCP holding a rows x ceil(cols/cs) column slab:
// the slab and the panel reflectors (ld = rows | 1), F (QB_NB per slab column), the pivot
// column, QB_NB dot products, two partial-norm arrays, the replicated permutation and the
// slab's column positions.
__host__ __device__ inline long long qb_need(int rows, int cols, int cs, int elem) {
    const long long cpc = (cols + cs - 1) / cs;
    const long long ld = rows | 1;
    return (ld * cpc + ld * QB_NB + cpc * QB_NB + rows + QB_NB + 2 * cpc) * elem + ((long long)cols + cpc) * 4;
}

// Gather columns [c0, c1) of the sparsification matrix Asn = [A_sn | A_ns^T] of item `it`
// (src/tree.cpp:1189-1224: the in-edge blocks as they are, the out-edge blocks
// transposed, in the plan's piece order) into A (column j - c0 at A + (j - c0) * lda).
template <typename T>
__device__ inline void qc_gather_slab(const Ctx<T>& c, const DSpars& it, const DAsn* __restrict__ pieces, int rows,
                                      int c0, int c1, T* A, int lda) {
    const int tid = threadIdx.x, nth = blockDim.x;
    int col = 0;
    for (int p = 0; p < it.count && col < c1; p++) {
        const DAsn pc = pieces[it.first + p];
        const int n = c.csize[pc.nbr];
        const int lo = max(col, c0), hi = min(col + n, c1);
        if (lo < hi) {
            const T* B = bptr(c, pc.block);
            const int bld = c.blk[pc.block].ld;
            const int width = hi - lo;
            if (!pc.transposed) {
                for (int idx = tid; idx < rows * width; idx += nth) {
                    const int i = idx % rows, jj = idx / rows;
                    A[i + (size_t)(lo - c0 + jj) * lda] = B[i + (size_t)(lo - col + jj) * bld];
                }
            } else {
                for (int idx = tid; idx < rows * width; idx += nth) {
                    const int jj = idx % width, i = idx / width;
                    A[i + (size_t)(lo - c0 + jj) * lda] = B[(lo - col + jj) + (size_t)i * bld];
                }
            }
        }
        col += n;
    }
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
//  dynamic shared bytes, vec_rows, projection); vec_rows: slabs of at least that many rows
//  take the vectorised trailing update (INT_MAX: none)
template <typename T>
using QcKernel = void (*)(Ctx<T>, const DSpars*, const DAsn*, T*, T*, int*, int*, T*, int*, int*, int*, double,
                          int, int, QcProj<T>);

// column slabs in the cluster's shared memory, for CTAs of `threads` threads (at most
// QC_THREADS, or at most QC_WIDE_THREADS)
template <typename T>
QcKernel<T> qrcp_smem_kernel_ptr(int threads = QC_THREADS);
// column slabs in global memory, for the matrices the shared-memory launch flagged
template <typename T>
QcKernel<T> qrcp_gslab_kernel_ptr();
// the blocked (panel) variant with slabs in shared memory, for matrices of at most
// 32 * rpl rows (rpl in 1, 2, 4, 8, 12; nullptr otherwise); plain QRCP only (no projection)
template <typename T>
QcKernel<T> qrcp_blocked_kernel_ptr(int rpl);

}  // namespace spand

// CUDA kernels and the device driver of the GB300 spaND factorization and solve.
//
// Every kernel reads cluster sizes from device memory (csize: current size, rows0: size
// when the cluster's hierarchy level started).  Work lists are uploaded once from the
// symbolic plan; grids are sized from capacities and surplus blocks exit early.
// Citations are path:line into leopoldcambier/spaND_public.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

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

template <typename T>
__device__ T warp_sum(T v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ------------------------------------------------------------------------------------
// Cholesky of pivot blocks, one block per pivot (dpotrf 'L', tree.cpp:582-593)
// Right-looking, column by column; the block is staged in shared memory when it fits.
// ------------------------------------------------------------------------------------
template <typename T>
__global__ void potrf_kernel(Ctx<T> c, const int* __restrict__ pivots, const int* __restrict__ clusters, int count,
                             int smem_elems) {
    extern __shared__ unsigned char smem_raw[];
    T* sm = reinterpret_cast<T*>(smem_raw);
    const int item = blockIdx.x;
    if (item >= count) return;
    // Another block of this launch may record a failure at any time: read the status
    // once per block so that every thread takes the same branch.
    __shared__ int failed;
    if (threadIdx.x == 0) failed = *(volatile int*)&c.status->not_spd;
    __syncthreads();
    if (failed) return;
    const int cl = clusters[item];
    const int n = c.csize[cl];
    if (n == 0) return;
    T* G = bptr(c, pivots[item]);
    const int gld = c.blk[pivots[item]].ld;
    const bool in_smem = (long long)n * n <= smem_elems;
    T* A = in_smem ? sm : G;
    const int ld = in_smem ? n : gld;
    if (in_smem) {
        for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
            int i = idx % n, j = idx / n;
            sm[i + j * n] = G[i + (size_t)j * gld];
        }
    }
    __shared__ T dshared;
    __shared__ int bad;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    for (int j = 0; j < n; j++) {
        if (threadIdx.x == 0) {
            T ajj = A[j + (size_t)j * ld];
            if (!(ajj > T(0))) {
                bad = 1;
                dshared = T(1);
            } else {
                dshared = dsqrt(ajj);
            }
            A[j + (size_t)j * ld] = dshared;
        }
        __syncthreads();
        if (bad) break;
        const T d = dshared;
        const T inv = T(1) / d;
        for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) A[i + (size_t)j * ld] *= inv;
        __syncthreads();
        // trailing lower update: A[i,k] -= A[i,j] A[k,j], j < k <= i
        const int m = n - j - 1;
        for (int idx = threadIdx.x; idx < m * m; idx += blockDim.x) {
            int ii = idx % m, kk = idx / m;
            if (ii < kk) continue;
            int i = j + 1 + ii, k = j + 1 + kk;
            A[i + (size_t)k * ld] -= A[i + (size_t)j * ld] * A[k + (size_t)j * ld];
        }
        __syncthreads();
    }
    if (bad) {
        if (threadIdx.x == 0) atomicCAS(&c.status->not_spd, 0, cl + 1);
        return;
    }
    if (in_smem) {
        for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
            int i = idx % n, j = idx / n;
            G[i + (size_t)j * gld] = sm[i + j * n];
        }
    }
}

// ------------------------------------------------------------------------------------
// Triangular solves of edge blocks with a cluster's Cholesky factor (tree.cpp:640-663)
// side 1: B (m x n) <- B L^{-T}; one thread per row of B.
// side 0: B (n x m) <- L^{-1} B; one warp per column of B.
// ------------------------------------------------------------------------------------
constexpr int TRSM_ROWS = 128;   // rows of B per block, side 1
constexpr int TRSM_COLS = 16;    // columns of B per block, side 0 (one warp each, 16 warps)

template <typename T>
__global__ void trsm_kernel(Ctx<T> c, const DTrsm* __restrict__ items, const DTile* __restrict__ tiles, int ntiles) {
    const int t = blockIdx.x;
    if (t >= ntiles || c.status->not_spd) return;
    const DTrsm it = items[tiles[t].item];
    const int n = c.csize[it.cluster];
    if (n == 0) return;
    const T* L = bptr(c, it.lblock);
    const int lld = c.blk[it.lblock].ld;
    T* B = bptr(c, it.block);
    const int bld = c.blk[it.block].ld;
    if (it.side == 1) {
        const int m = c.csize[c.blk[it.block].rowc];
        const int r = tiles[t].tile_i * TRSM_ROWS + threadIdx.x;
        if (r >= m) return;
        T* row = B + r;
        for (int j = 0; j < n; j++) {
            const T x = row[(size_t)j * bld] / L[j + (size_t)j * lld];
            row[(size_t)j * bld] = x;
            const T* lj = L + (size_t)j * lld;
            for (int k = j + 1; k < n; k++) row[(size_t)k * bld] -= x * lj[k];
        }
    } else {
        const int m = c.csize[c.blk[it.block].colc];
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        const int col = tiles[t].tile_i * TRSM_COLS + w;
        if (col >= m) return;
        T* b = B + (size_t)col * bld;
        for (int k = 0; k < n; k++) {
            const T x = b[k] / L[k + (size_t)k * lld];
            __syncwarp();
            if (lane == 0) b[k] = x;
            const T* lk = L + (size_t)k * lld;
            for (int i = k + 1 + lane; i < n; i += 32) b[i] -= lk[i] * x;
            __syncwarp();
        }
    }
}

// ------------------------------------------------------------------------------------
// Schur complement updates grouped by target block, applied in the reference order
// (tree.cpp:748-793, 858-883): C(n1 x n2) -= op1(B1) op2(B2).  32x32 output tile per
// block, 256 threads, 2x2 outputs per thread, K staged through shared memory.
// ------------------------------------------------------------------------------------
constexpr int ST = 32;
constexpr int SK = 16;

template <typename T>
__global__ void __launch_bounds__(256) schur_kernel(Ctx<T> c, const DTarget* __restrict__ targets,
                                                     const DUpd* __restrict__ ups, const DTile* __restrict__ tiles,
                                                     int ntiles) {
    const int t = blockIdx.x;
    if (t >= ntiles || c.status->not_spd) return;
    const DTarget tg = targets[tiles[t].item];
    const DBlock cb = c.blk[tg.target];
    const int M = c.csize[cb.rowc], N = c.csize[cb.colc];
    const int i0 = tiles[t].tile_i * ST, j0 = tiles[t].tile_j * ST;
    if (i0 >= M || j0 >= N) return;
    if (tg.syrk && i0 + ST <= j0) return;  // strictly upper tile
    __shared__ T Xs[ST][SK + 1];
    __shared__ T Ys[SK][ST + 1];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    T* C = c.arena + cb.off;
    const int ldc = cb.ld;
    T acc[2][2];
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 2; b++) {
            int i = i0 + tx + 16 * a, j = j0 + ty + 16 * b;
            acc[a][b] = (i < M && j < N) ? C[i + (size_t)j * ldc] : T(0);
        }
    for (int u = 0; u < tg.count; u++) {
        const DUpd up = ups[tg.first + u];
        const int S = c.csize[up.s];
        const T* B1 = bptr(c, up.b1);
        const int ld1 = c.blk[up.b1].ld;
        const T* B2 = bptr(c, up.b2);
        const int ld2 = c.blk[up.b2].ld;
        for (int k0 = 0; k0 < S; k0 += SK) {
            // X tile: ST x SK, X[i,k] = t1 ? B1[k + i ld1] : B1[i + k ld1]
            for (int idx = threadIdx.x; idx < ST * SK; idx += 256) {
                int ii, kk;
                if (up.t1) { kk = idx % SK; ii = idx / SK; } else { ii = idx % ST; kk = idx / ST; }
                int i = i0 + ii, k = k0 + kk;
                T v = T(0);
                if (i < M && k < S) v = up.t1 ? B1[k + (size_t)i * ld1] : B1[i + (size_t)k * ld1];
                Xs[ii][kk] = v;
            }
            // Y tile: SK x ST, Y[k,j] = t2 ? B2[j + k ld2] : B2[k + j ld2]
            for (int idx = threadIdx.x; idx < ST * SK; idx += 256) {
                int jj, kk;
                if (up.t2) { jj = idx % ST; kk = idx / ST; } else { kk = idx % SK; jj = idx / SK; }
                int j = j0 + jj, k = k0 + kk;
                T v = T(0);
                if (j < N && k < S) v = up.t2 ? B2[j + (size_t)k * ld2] : B2[k + (size_t)j * ld2];
                Ys[kk][jj] = v;
            }
            __syncthreads();
            const int kmax = min(SK, S - k0);
            for (int kk = 0; kk < kmax; kk++) {
                T x0 = Xs[tx][kk], x1 = Xs[tx + 16][kk];
                T y0 = Ys[kk][ty], y1 = Ys[kk][ty + 16];
                acc[0][0] -= x0 * y0;
                acc[1][0] -= x1 * y0;
                acc[0][1] -= x0 * y1;
                acc[1][1] -= x1 * y1;
            }
            __syncthreads();
        }
    }
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 2; b++) {
            int i = i0 + tx + 16 * a, j = j0 + ty + 16 * b;
            if (i < M && j < N && (!tg.syrk || i >= j)) C[i + (size_t)j * ldc] = acc[a][b];
        }
}

// ------------------------------------------------------------------------------------
// Sparsification (tree.cpp:1189-1224, 1292-1347, 980-1104)
// ------------------------------------------------------------------------------------
// Asn = [A_sn (in-edges) | A_ns^T (out-edges)], rows = size(c); ld = cap(c).
template <typename T>
__global__ void asn_gather_kernel(Ctx<T> c, const DSpars* __restrict__ items, const DAsn* __restrict__ pieces, T* ws,
                                  int* colcount) {
    if (c.status->not_spd) return;
    const DSpars it = items[blockIdx.x];
    const int rows = c.csize[it.cluster];
    const int ld = c.cap[it.cluster];
    T* W = ws + it.ws_off;
    int col = 0;
    for (int p = 0; p < it.count; p++) {
        const DAsn pc = pieces[it.first + p];
        const int n = c.csize[pc.nbr];
        const T* B = bptr(c, pc.block);
        const int bld = c.blk[pc.block].ld;
        if (!pc.transposed) {
            for (int idx = threadIdx.x; idx < rows * n; idx += blockDim.x) {
                int i = idx % rows, j = idx / rows;
                W[i + (size_t)(col + j) * ld] = B[i + (size_t)j * bld];
            }
        } else {
            for (int idx = threadIdx.x; idx < rows * n; idx += blockDim.x) {
                int j = idx % n, i = idx / n;
                W[i + (size_t)(col + j) * ld] = B[j + (size_t)i * bld];
            }
        }
        col += n;
    }
    if (threadIdx.x == 0) colcount[blockIdx.x] = col;
}

// Relative window inside which partial column norms count as tied (same rule as the
// oracle's restated dgeqp3).
template <typename T>
__device__ __forceinline__ T qrcp_tie() {
    return sizeof(T) == 8 ? T(1e-7) : T(1e-4);
}

// Householder QR with column pivoting (LAPACK dgeqp3/dlaqp2 with LAWN 176 norm
// downdating), stopped as soon as |R_ii| / |R_00| < tol (choose_rank, util.cpp:434-452).
// One block per matrix; the matrix stays in global memory (L2), reflector in shared.
template <typename T>
__global__ void __launch_bounds__(512) qrcp_kernel(Ctx<T> c, const DSpars* __restrict__ items, T* ws, T* norms,
                                                    int* jpvt_ws, const int* __restrict__ colcount, T* taus,
                                                    int* rank_out, double tol) {
    extern __shared__ unsigned char smem_raw[];
    T* vsh = reinterpret_cast<T*>(smem_raw);  // cap(c) entries
    __shared__ T red[33];
    __shared__ T s_val[16];
    __shared__ int s_idx[16];
    __shared__ int s_pvt;
    __shared__ T s_beta, s_tau, s_scal;
    __shared__ int s_stop;
    if (c.status->not_spd) return;
    const DSpars it = items[blockIdx.x];
    const int rows = c.csize[it.cluster];
    const int cols = colcount[blockIdx.x];
    const int ld = c.cap[it.cluster];
    T* A = ws + it.ws_off;
    T* vn1 = norms + 2 * it.col_off;
    T* vn2 = vn1 + it.cap_cols;
    int* jpvt = jpvt_ws + it.col_off;
    T* tau = taus + it.tau_off;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int mn = min(rows, cols);
    int rank;
    if (tol >= 1.0) {
        // choose_rank returns 0 without looking at R; keep the pivot vector defined
        rank = 0;
        for (int j = threadIdx.x; j < cols; j += blockDim.x) jpvt[j] = j;
    } else {
        // initial column norms, warp per column
        for (int j = w; j < cols; j += nw) {
            T s = 0;
            const T* a = A + (size_t)j * ld;
            for (int r = lane; r < rows; r += 32) s += a[r] * a[r];
            s = warp_sum(s);
            if (lane == 0) {
                vn1[j] = dsqrt(s);
                vn2[j] = vn1[j];
                jpvt[j] = j;
            }
        }
        const T tol3z = dsqrt(sizeof(T) == 8 ? T(2.220446049250313e-16) : T(1.1920929e-07));
        T r00 = 0;
        rank = mn;
        if (threadIdx.x == 0) s_stop = 0;
        __syncthreads();
        for (int i = 0; i < mn; i++) {
            // pivot: first column of [i, cols) whose partial norm is within a relative
            // qrcp_tie<T>() of the largest; exact-arithmetic ties (mirror-symmetric
            // stencil columns) then do not depend on the summation order of the norms.
            T bv = 0;
            for (int j = i + threadIdx.x; j < cols; j += blockDim.x) bv = fmax(bv, vn1[j]);
            for (int o = 16; o > 0; o >>= 1) bv = fmax(bv, __shfl_xor_sync(0xffffffffu, bv, o));
            if (lane == 0) s_val[w] = bv;
            __syncthreads();
            T vmax = s_val[0];
            for (int k = 1; k < nw; k++) vmax = fmax(vmax, s_val[k]);
            const T thresh = vmax * (T(1) - qrcp_tie<T>());
            int bi = cols;
            for (int j = i + threadIdx.x; j < cols; j += blockDim.x)
                if (vn1[j] >= thresh) { bi = j; break; }
            for (int o = 16; o > 0; o >>= 1) bi = min(bi, __shfl_xor_sync(0xffffffffu, bi, o));
            if (lane == 0) s_idx[w] = bi;
            __syncthreads();
            if (threadIdx.x == 0) {
                int id = s_idx[0];
                for (int k = 1; k < nw; k++) id = min(id, s_idx[k]);
                s_pvt = id < cols ? id : i;  // all norms NaN: keep the current column
            }
            __syncthreads();
            const int pvt = s_pvt;
            if (pvt != i) {
                T* a = A + (size_t)i * ld;
                T* b = A + (size_t)pvt * ld;
                for (int r = threadIdx.x; r < rows; r += blockDim.x) {
                    T tmp = a[r];
                    a[r] = b[r];
                    b[r] = tmp;
                }
                if (threadIdx.x == 0) {
                    int tj = jpvt[i];
                    jpvt[i] = jpvt[pvt];
                    jpvt[pvt] = tj;
                    vn1[pvt] = vn1[i];
                    vn2[pvt] = vn2[i];
                }
            }
            __syncthreads();
            // reflector of column i (dlarfg)
            T* ai = A + (size_t)i * ld;
            T part = 0;
            for (int r = i + 1 + threadIdx.x; r < rows; r += blockDim.x) part += ai[r] * ai[r];
            T xnorm2 = block_sum(part, red);
            if (threadIdx.x == 0) {
                T alpha = ai[i];
                T xnorm = dsqrt(xnorm2);
                T beta, tu, sc;
                if (xnorm == T(0)) {
                    beta = alpha;
                    tu = 0;
                    sc = 0;
                } else {
                    beta = -copysign(hypot(alpha, xnorm), alpha);
                    tu = (beta - alpha) / beta;
                    sc = T(1) / (alpha - beta);
                }
                s_beta = beta;
                s_tau = tu;
                s_scal = sc;
                T rii = fabs(beta);
                if (i == 0) r00 = rii;
                int stop = 0;
                if (tol != 0.0 && i >= 1) {
                    T ratio = rii / r00;
                    if (!(ratio >= T(tol))) stop = 1;
                }
                s_stop = stop;
                red[32] = r00;
            }
            __syncthreads();
            r00 = red[32];
            if (s_stop) {
                rank = i;
                break;
            }
            const T tu = s_tau, sc = s_scal;
            if (tu != T(0))
                for (int r = i + 1 + threadIdx.x; r < rows; r += blockDim.x) ai[r] *= sc;
            __syncthreads();
            if (threadIdx.x == 0) {
                ai[i] = s_beta;
                tau[i] = tu;
            }
            for (int r = i + 1 + threadIdx.x; r < rows; r += blockDim.x) vsh[r] = ai[r];
            if (threadIdx.x == 0) vsh[i] = T(1);
            __syncthreads();
            // apply H(i) to the trailing columns and downdate their norms, warp per column
            for (int j = i + 1 + w; j < cols; j += nw) {
                T* aj = A + (size_t)j * ld;
                if (tu != T(0)) {
                    T s = 0;
                    for (int r = i + lane; r < rows; r += 32) s += vsh[r] * aj[r];
                    s = warp_sum(s) * tu;
                    for (int r = i + lane; r < rows; r += 32) aj[r] -= s * vsh[r];
                }
                __syncwarp();
                T v1 = vn1[j];
                if (v1 != T(0)) {
                    T temp = fabs(aj[i]) / v1;
                    temp = T(1) - temp * temp;
                    temp = temp > T(0) ? temp : T(0);
                    T rr = v1 / vn2[j];
                    T temp2 = temp * rr * rr;
                    if (temp2 <= tol3z) {
                        T s = 0;
                        for (int r = i + 1 + lane; r < rows; r += 32) s += aj[r] * aj[r];
                        s = warp_sum(s);
                        if (lane == 0) {
                            if (i < rows - 1) {
                                vn1[j] = dsqrt(s);
                                vn2[j] = vn1[j];
                            } else {
                                vn1[j] = 0;
                                vn2[j] = 0;
                            }
                        }
                    } else if (lane == 0) {
                        vn1[j] = v1 * dsqrt(temp);
                    }
                }
                __syncwarp();
            }
            __syncthreads();
        }
    }
    if (threadIdx.x == 0) rank_out[it.cluster] = rank;
}

// Compressed edges AsnP = triu(R[:k,:]) P^T written back into the cluster's edge blocks,
// reflectors saved for the Orthogonal op, cluster size set to the rank.
template <typename T>
__global__ void sparsify_scatter_kernel(Ctx<T> c, const DSpars* __restrict__ items, const DAsn* __restrict__ pieces,
                                        const T* ws, int* jpvt_ws, int* ipvt_ws, const int* __restrict__ rank_in,
                                        T* vstore, const T* taus_ws, T* taustore, const int* __restrict__ colcount) {
    if (c.status->not_spd) return;
    const DSpars it = items[blockIdx.x];
    const int rows = c.csize[it.cluster];
    const int k = rank_in[it.cluster];
    if (k >= rows) return;
    const int cols = colcount[blockIdx.x];
    const int ld = c.cap[it.cluster];
    const T* A = ws + it.ws_off;
    const int* jpvt = jpvt_ws + it.col_off;
    int* ipvt = ipvt_ws + it.col_off;
    if (k > 0)
        for (int j = threadIdx.x; j < cols; j += blockDim.x) {
            const int q = jpvt[j];
            if (q >= 0 && q < cols) ipvt[q] = j;
        }
    T* V = vstore + it.v_off;
    for (int idx = threadIdx.x; idx < rows * k; idx += blockDim.x) {
        int i = idx % rows, j = idx / rows;
        V[i + (size_t)j * ld] = A[i + (size_t)j * ld];
    }
    for (int j = threadIdx.x; j < k; j += blockDim.x) taustore[it.tau_off + j] = taus_ws[it.tau_off + j];
    __syncthreads();
    int col = 0;
    for (int p = 0; p < it.count; p++) {
        const DAsn pc = pieces[it.first + p];
        const int n = c.csize[pc.nbr];
        T* B = bptr(c, pc.block);
        const int bld = c.blk[pc.block].ld;
        for (int idx = threadIdx.x; idx < k * n; idx += blockDim.x) {
            int i, jj;
            if (!pc.transposed) { i = idx % k; jj = idx / k; } else { jj = idx % n; i = idx / n; }
            const int q = ipvt[col + jj];
            const T v = (i <= q) ? A[i + (size_t)q * ld] : T(0);
            if (!pc.transposed) B[i + (size_t)jj * bld] = v;
            else B[jj + (size_t)i * bld] = v;
        }
        col += n;
    }
    __syncthreads();
    if (threadIdx.x == 0) c.csize[it.cluster] = k;
}

// ------------------------------------------------------------------------------------
// Merge (tree.cpp:1106-1184)
// ------------------------------------------------------------------------------------
__global__ void merge_sizes_kernel(int* csize, int* rows0, int* cpos, const int* __restrict__ parents, int np,
                                   const int* __restrict__ child_ptr, const int* __restrict__ child_idx) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    int pos = 0;
    for (int k = child_ptr[p]; k < child_ptr[p + 1]; k++) {
        int ch = child_idx[k];
        cpos[ch] = pos;
        pos += csize[ch];
    }
    csize[parents[p]] = pos;
    rows0[parents[p]] = pos;
}

constexpr int MT = 32;

template <typename T>
__global__ void merge_copy_kernel(Ctx<T> c, const DMerge* __restrict__ items, const DTile* __restrict__ tiles,
                                  int ntiles, const int* __restrict__ cpos) {
    const int t = blockIdx.x;
    if (t >= ntiles || c.status->not_spd) return;
    const DMerge m = items[tiles[t].item];
    const int R = c.csize[m.nold], Cn = c.csize[m.sold];
    const int i0 = tiles[t].tile_i * MT, j0 = tiles[t].tile_j * MT;
    if (i0 >= R || j0 >= Cn) return;
    const DBlock db = c.blk[m.dst];
    T* D = c.arena + db.off + cpos[m.nold] + (size_t)cpos[m.sold] * db.ld;
    const DBlock sb = c.blk[m.src];
    const bool ident = sb.flag == BLK_IDENTITY;
    const T* S = ident ? nullptr : c.arena + sb.off;
    for (int idx = threadIdx.x; idx < MT * MT; idx += blockDim.x) {
        int i = i0 + idx % MT, j = j0 + idx / MT;
        if (i < R && j < Cn) D[i + (size_t)j * db.ld] = ident ? T(i == j) : S[i + (size_t)j * sb.ld];
    }
}

__global__ void snapshot_kernel(const int* csize, int* rows0, const int* __restrict__ clusters, int n) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) rows0[clusters[k]] = csize[clusters[k]];
}

// ------------------------------------------------------------------------------------
// Solve kernels (tree.cpp:1610-1635, operations.cpp:31-208).  x slots: xs[xoff[c] + i
// + r * xld], r < nrhs.
// ------------------------------------------------------------------------------------
template <typename T>
struct XCtx {
    T* xs;
    long long xld;
    const long long* xoff;
    int nrhs;
};

// b = P^T x (natural -> permuted leaf slots), FP64 in, T out
template <typename T>
__global__ void perm_in_kernel(const double* __restrict__ x, int ldx, XCtx<T> X, const int* __restrict__ perm,
                               const long long* __restrict__ slot, int n) {
    long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k >= (long long)n * X.nrhs) return;
    int p = (int)(k % n), r = (int)(k / n);
    X.xs[slot[p] + r * X.xld] = (T)x[perm[p] + (size_t)r * ldx];
}

template <typename T>
__global__ void perm_out_kernel(double* __restrict__ x, int ldx, XCtx<T> X, const int* __restrict__ perm,
                                const long long* __restrict__ slot, int n) {
    long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k >= (long long)n * X.nrhs) return;
    int p = (int)(k % n), r = (int)(k / n);
    x[perm[p] + (size_t)r * ldx] = (double)X.xs[slot[p] + r * X.xld];
}

// x <- L^{-1} x (fwd) or L^{-T} x (bwd), ScalingLLT (operations.cpp:97-103)
template <typename T>
__global__ void trsv_kernel(Ctx<T> c, XCtx<T> X, const int* __restrict__ clusters, const int* __restrict__ lblocks,
                            int count, int trans) {
    const int item = blockIdx.x % count;
    const int r = blockIdx.x / count;
    const int cl = clusters[item];
    const int n = c.rows0[cl];
    if (n == 0) return;
    const T* L = bptr(c, lblocks[item]);
    const int ld = c.blk[lblocks[item]].ld;
    T* x = X.xs + X.xoff[cl] + r * X.xld;
    extern __shared__ unsigned char smem_raw[];
    T* xsh = reinterpret_cast<T*>(smem_raw);
    __shared__ T red[33];
    for (int i = threadIdx.x; i < n; i += blockDim.x) xsh[i] = x[i];
    __syncthreads();
    if (!trans) {
        for (int k = 0; k < n; k++) {
            const T xk = xsh[k] / L[k + (size_t)k * ld];
            __syncthreads();
            if (threadIdx.x == 0) xsh[k] = xk;
            const T* lk = L + (size_t)k * ld;
            for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) xsh[i] -= lk[i] * xk;
            __syncthreads();
        }
    } else {
        for (int k = n - 1; k >= 0; k--) {
            const T* lk = L + (size_t)k * ld;
            T part = 0;
            for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) part += lk[i] * xsh[i];
            T s = block_sum(part, red);
            if (threadIdx.x == 0) xsh[k] = (xsh[k] - s) / lk[k];
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = xsh[i];
}

// Forward Gemm ops grouped by neighbour: x_n -= A_ns x_s (GemmSymmOut) or A_sn^T x_s (GemmSymmIn)
template <typename T>
__global__ void gemm_fwd_kernel(Ctx<T> c, XCtx<T> X, const DGroup* __restrict__ groups, const DGemmOp* __restrict__ ops,
                                int ngroups) {
    const int g = blockIdx.x % ngroups;
    const int r = blockIdx.x / ngroups;
    const DGroup G = groups[g];
    const int nb = G.key;
    const int nn = c.rows0[nb];
    T* xn = X.xs + X.xoff[nb] + r * X.xld;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int o = 0; o < G.count; o++) {
        const DGemmOp op = ops[G.first + o];
        const int ns = c.csize[op.self];
        const T* xs = X.xs + X.xoff[op.self] + r * X.xld;
        const T* A = bptr(c, op.block);
        const int ld = c.blk[op.block].ld;
        if (op.kind == 1) {
            for (int i = threadIdx.x; i < nn; i += blockDim.x) {
                T s = 0;
                for (int j = 0; j < ns; j++) s += A[i + (size_t)j * ld] * xs[j];
                xn[i] -= s;
            }
        } else {
            for (int i = w; i < nn; i += nw) {
                const T* a = A + (size_t)i * ld;
                T s = 0;
                for (int j = lane; j < ns; j += 32) s += a[j] * xs[j];
                s = warp_sum(s);
                if (lane == 0) xn[i] -= s;
            }
        }
        __syncthreads();
    }
}

// Backward Gemm ops grouped by eliminated cluster: x_s -= A_ns^T x_n or A_sn x_n
template <typename T>
__global__ void gemm_bwd_kernel(Ctx<T> c, XCtx<T> X, const DGroup* __restrict__ groups, const DGemmOp* __restrict__ ops,
                                int ngroups) {
    const int g = blockIdx.x % ngroups;
    const int r = blockIdx.x / ngroups;
    const DGroup G = groups[g];
    const int sc = G.key;
    const int ns = c.csize[sc];
    T* xs = X.xs + X.xoff[sc] + r * X.xld;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int o = 0; o < G.count; o++) {
        const DGemmOp op = ops[G.first + o];
        const int nn = c.rows0[op.nbr];
        const T* xn = X.xs + X.xoff[op.nbr] + r * X.xld;
        const T* A = bptr(c, op.block);
        const int ld = c.blk[op.block].ld;
        if (op.kind == 1) {
            for (int i = w; i < ns; i += nw) {
                const T* a = A + (size_t)i * ld;
                T s = 0;
                for (int j = lane; j < nn; j += 32) s += a[j] * xn[j];
                s = warp_sum(s);
                if (lane == 0) xs[i] -= s;
            }
        } else {
            for (int i = threadIdx.x; i < ns; i += blockDim.x) {
                T s = 0;
                for (int j = 0; j < nn; j++) s += A[i + (size_t)j * ld] * xn[j];
                xs[i] -= s;
            }
        }
        __syncthreads();
    }
}

// Orthogonal op: x <- Q^T x (fwd) or Q x (bwd), k = rank reflectors (operations.cpp:153-158)
template <typename T>
__global__ void ortho_kernel(Ctx<T> c, XCtx<T> X, const DOrtho* __restrict__ items, int count, const T* vstore,
                             const T* taustore, int trans) {
    const int item = blockIdx.x % count;
    const int r = blockIdx.x / count;
    const DOrtho it = items[item];
    const int rows = c.rows0[it.cluster];
    const int k = c.csize[it.cluster];
    if (k >= rows) return;
    const int ld = c.cap[it.cluster];
    const T* V = vstore + it.v_off;
    const T* tau = taustore + it.tau_off;
    T* x = X.xs + X.xoff[it.cluster] + r * X.xld;
    extern __shared__ unsigned char smem_raw[];
    T* xsh = reinterpret_cast<T*>(smem_raw);
    __shared__ T red[33];
    for (int i = threadIdx.x; i < rows; i += blockDim.x) xsh[i] = x[i];
    __syncthreads();
    for (int q = 0; q < k; q++) {
        const int i = trans ? q : k - 1 - q;
        const T* v = V + (size_t)i * ld;
        T part = 0;
        for (int rr = i + 1 + threadIdx.x; rr < rows; rr += blockDim.x) part += v[rr] * xsh[rr];
        T s = block_sum(part, red);
        s = (s + xsh[i]) * tau[i];
        __syncthreads();
        if (threadIdx.x == 0) xsh[i] -= s;
        for (int rr = i + 1 + threadIdx.x; rr < rows; rr += blockDim.x) xsh[rr] -= s * v[rr];
        __syncthreads();
    }
    for (int i = threadIdx.x; i < rows; i += blockDim.x) x[i] = xsh[i];
}

// Merge op: parent x = children heads concatenated (fwd) and back (bwd)
template <typename T>
__global__ void merge_x_kernel(Ctx<T> c, XCtx<T> X, const int* __restrict__ children, const int* __restrict__ parent_of,
                               int nchildren, const int* __restrict__ cpos, int fwd) {
    const int k = blockIdx.x % nchildren;
    const int r = blockIdx.x / nchildren;
    const int ch = children[k];
    const int p = parent_of[k];
    const int n = c.csize[ch];
    T* xc = X.xs + X.xoff[ch] + r * X.xld;
    T* xp = X.xs + X.xoff[p] + cpos[ch] + r * X.xld;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        if (fwd) xp[i] = xc[i];
        else xc[i] = xp[i];
    }
}

// ------------------------------------------------------------------------------------
// FP64 Krylov kernels
// ------------------------------------------------------------------------------------
__global__ void spmv_kernel(int n, const int* __restrict__ rp, const int* __restrict__ ci, const double* __restrict__ v,
                            const double* __restrict__ x, double* __restrict__ y) {
    int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n) return;
    double s = 0;
    for (int k = rp[row]; k < rp[row + 1]; k++) s += v[k] * x[ci[k]];
    y[row] = s;
}

constexpr int RED_BLOCKS = 304;  // 2 x 152 SMs
constexpr int RED_THREADS = 512;

// partial[b] = sum over the block's strided range of a*b (fixed order)
__global__ void dot_partial_kernel(int n, const double* __restrict__ a, const double* __restrict__ b, double* partial) {
    __shared__ double red[33];
    double s = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        s += a[i] * b[i];
    s = block_sum(s, red);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

__global__ void dot_final_kernel(const double* partial, int np, double* out) {
    __shared__ double red[33];
    double s = 0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) s += partial[i];
    s = block_sum(s, red);
    if (threadIdx.x == 0) *out = s;
}

// scalars: [0] absNew [1] p.Ap [2] r.r [3] absOld
__global__ void cg_update_xr_kernel(int n, double* x, double* r, const double* p, const double* Ap, const double* sc) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double alpha = sc[0] / sc[1];
    x[i] += alpha * p[i];
    r[i] -= alpha * Ap[i];
}

__global__ void cg_update_p_kernel(int n, double* p, const double* z, const double* sc) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double beta = sc[0] / sc[3];
    p[i] = z[i] + beta * p[i];
}

__global__ void copy_scalar_kernel(double* sc, int dst, int src) { sc[dst] = sc[src]; }

__global__ void sub_kernel(int n, const double* a, const double* b, double* y) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) y[i] = a[i] - b[i];
}

// ------------------------------------------------------------------------------------
// Kernel profiler
// ------------------------------------------------------------------------------------
KernelProfiler::~KernelProfiler() {
    for (cudaEvent_t e : pool_) cudaEventDestroy(e);
}

cudaEvent_t KernelProfiler::take() {
    if (used_ == pool_.size()) {
        cudaEvent_t e;
        SPAND_CUDA(cudaEventCreate(&e));
        pool_.push_back(e);
    }
    return pool_[used_++];
}

void KernelProfiler::begin(cudaStream_t s, const char* cls) {
    if (!on_) return;
    cur_ = cls;
    cur_a_ = take();
    SPAND_CUDA(cudaEventRecord(cur_a_, s));
}

void KernelProfiler::end(cudaStream_t s) {
    if (!on_) return;
    cudaEvent_t b = take();
    SPAND_CUDA(cudaEventRecord(b, s));
    recs_.push_back({cur_, cur_a_, b});
}

void KernelProfiler::collect() {
    for (const Rec& r : recs_) {
        SPAND_CUDA(cudaEventSynchronize(r.b));
        float ms = 0;
        SPAND_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
        auto it = std::find_if(totals_.begin(), totals_.end(), [&](const Entry& e) { return e.cls == r.cls; });
        if (it == totals_.end()) {
            totals_.push_back({r.cls, 0, 0.0});
            it = totals_.end() - 1;
        }
        it->launches++;
        it->ms += ms;
    }
    recs_.clear();
    used_ = 0;
}

void KernelProfiler::clear() {
    recs_.clear();
    used_ = 0;
    totals_.clear();
}

// ------------------------------------------------------------------------------------
// Host driver
// ------------------------------------------------------------------------------------
template <typename V>
static V* dev_upload(const std::vector<V>& h, std::vector<void*>& owned, size_t& bytes, cudaStream_t s) {
    if (h.empty()) return nullptr;
    V* d = nullptr;
    SPAND_CUDA(cudaMalloc(&d, h.size() * sizeof(V)));
    owned.push_back(d);
    bytes += h.size() * sizeof(V);
    SPAND_CUDA(cudaMemcpyAsync(d, h.data(), h.size() * sizeof(V), cudaMemcpyHostToDevice, s));
    SPAND_CUDA(cudaStreamSynchronize(s));
    return d;
}

static std::vector<DTile> tiles_1d(const std::vector<int>& extents, int tile) {
    std::vector<DTile> t;
    for (size_t i = 0; i < extents.size(); i++) {
        int n = (extents[i] + tile - 1) / tile;
        for (int k = 0; k < n; k++) t.push_back({(int)i, k, 0});
    }
    return t;
}

template <typename T>
class DeviceFactor : public DeviceFactorBase {
   public:
    DeviceFactor(cudaStream_t s, const std::vector<int>& perm) : s_(s), perm_h_(perm) {}
    ~DeviceFactor() override {
        if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
        if (graph_) cudaGraphDestroy(graph_);
        if (xs_) cudaFree(xs_);
        for (void* p : owned_) cudaFree(p);
    }

    int precision_bytes() const override { return sizeof(T); }
    cudaStream_t stream() const override { return s_; }
    size_t device_bytes() const override { return bytes_; }

    void upload(const Plan& P, const std::vector<double>& assembled) override {
        P_ = &P;
        nc_ = P.nclusters;
        arena_ = alloc<T>(P.arena_len);
        pristine_ = alloc<T>(P.assembled_len);
        upload_values(assembled);
        std::vector<DBlock> blk(P.blocks.size());
        for (size_t b = 0; b < P.blocks.size(); b++)
            blk[b] = {(long long)P.blocks[b].off, P.blocks[b].ld, P.blocks[b].rowc, P.blocks[b].colc, P.blocks[b].flag};
        d_blk_ = up(blk);
        d_cap_ = up(P.c_cap);
        csize_ = alloc<int>(nc_);
        rows0_ = alloc<int>(nc_);
        rank_ = alloc<int>(nc_);
        cpos_ = alloc<int>(nc_);
        status_ = alloc<DStatus>(1);
        vstore_ = alloc<T>(std::max<int64_t>(P.v_len, 1));
        taustore_ = alloc<T>(std::max<int64_t>(P.tau_len, 1));
        tauws_ = alloc<T>(std::max<int64_t>(P.tau_len, 1));
        ws_ = alloc<T>(std::max<int64_t>(P.ws_len, 1));
        {
            std::vector<DUpd> u;
            for (const SchurUpdate& su : P.schur_updates) u.push_back({su.b1, su.t1, su.b2, su.t2, su.s});
            d_ups_ = up(u);
            std::vector<DAsn> a;
            for (const AsnPiece& ap : P.asn_pieces) a.push_back({ap.block, ap.nbr, ap.transposed});
            pieces_ = up(a);
        }
        int64_t max_cols = 1;
        int max_items = 1;
        levels_.resize(P.nlevels);
        for (int l = 0; l < P.nlevels; l++) {
            const LevelPlan& L = P.levels[l];
            LevelDev& D = levels_[l];
            D.n_elim = (int)L.elim_clusters.size();
            D.elim_clusters = up(L.elim_clusters);
            D.elim_pivots = up(L.elim_pivots);
            D.elim_smem = smem_for(L.elim_clusters, P);
            build_trsm(L.elim_trsm, L.elim_pivots, L.elim_clusters, P, D.elim_trsm0, D.elim_trsm1);
            {
                std::vector<DTarget> tg;
                std::vector<DTile> tiles;
                for (int t = 0; t < L.schur_count; t++) {
                    const SchurTarget& st = P.schur_targets[L.schur_first + t];
                    tg.push_back({st.target, st.syrk, st.first, st.count});
                    const PlanBlock& B = P.blocks[st.target];
                    int ti = (P.c_cap[B.rowc] + ST - 1) / ST, tj = (P.c_cap[B.colc] + ST - 1) / ST;
                    for (int a = 0; a < ti; a++)
                        for (int b = 0; b < tj; b++)
                            if (!st.syrk || a >= b) tiles.push_back({t, a, b});
                }
                D.schur_targets = up(tg);
                D.schur_tiles = up(tiles);
                D.n_schur_tiles = (int)tiles.size();
            }
            D.scaled = L.scaled;
            D.n_scale = (int)L.scale_clusters.size();
            D.scale_clusters = up(L.scale_clusters);
            D.scale_pivots = up(L.scale_pivots);
            D.scale_smem = smem_for(L.scale_clusters, P);
            build_trsm(L.scale_trsm, L.scale_pivots, L.scale_clusters, P, D.scale_trsm0, D.scale_trsm1);
            {
                std::vector<int> all;
                for (int cl = 0; cl < nc_; cl++)
                    if (P.c_hlevel[cl] == l) all.push_back(cl);
                D.n_level = (int)all.size();
                D.level_clusters = up(all);
            }
            for (const auto& wave : L.waves) {
                WaveDev W;
                std::vector<DSpars> items;
                int64_t coloff = 0;
                int maxcap = 1;
                for (const SparsifyItem& it : wave) {
                    items.push_back({it.cluster, it.first, it.count, it.cap_cols, (long long)it.ws_off,
                                     (long long)coloff, (long long)it.v_off, (long long)it.tau_off});
                    coloff += std::max(it.cap_cols, 1);
                    maxcap = std::max(maxcap, P.c_cap[it.cluster]);
                }
                if ((int64_t)maxcap * (int64_t)sizeof(T) > 200 * 1024)
                    throw DeviceError{SPAND_ERR_UNSUPPORTED, "cluster too large for the QRCP kernel"};
                max_cols = std::max(max_cols, coloff);
                max_items = std::max(max_items, (int)items.size());
                W.n = (int)items.size();
                W.items = up(items);
                W.maxcap = maxcap;
                D.waves.push_back(W);
            }
            D.merged = L.merged;
            if (L.merged) {
                std::vector<int> cptr(1, 0), cidx, parent_of;
                for (int p : L.merge_parents) {
                    for (int ch : P.c_children[p]) {
                        cidx.push_back(ch);
                        parent_of.push_back(p);
                    }
                    cptr.push_back((int)cidx.size());
                }
                D.n_parents = (int)L.merge_parents.size();
                D.parents = up(L.merge_parents);
                D.child_ptr = up(cptr);
                D.child_idx = up(cidx);
                D.child_parent = up(parent_of);
                D.n_children = (int)cidx.size();
                std::vector<DMerge> mc;
                std::vector<DTile> tiles;
                for (size_t k = 0; k < L.merge_copies.size(); k++) {
                    const MergeCopy& m = L.merge_copies[k];
                    mc.push_back({m.src, m.dst, m.nold, m.sold});
                    int ti = (P.c_cap[m.nold] + MT - 1) / MT, tj = (P.c_cap[m.sold] + MT - 1) / MT;
                    for (int a = 0; a < ti; a++)
                        for (int b = 0; b < tj; b++) tiles.push_back({(int)k, a, b});
                }
                D.merge_items = up(mc);
                D.merge_tiles = up(tiles);
                D.n_merge_tiles = (int)tiles.size();
            }
            D.n_elim_llt = (int)L.op_elim_llt.size();
            D.elim_llt = up(L.op_elim_llt);
            D.elim_llt_blk = up(L.op_elim_llt_block);
            D.n_scale_llt = (int)L.op_scale_llt.size();
            D.scale_llt = up(L.op_scale_llt);
            D.scale_llt_blk = up(L.op_scale_llt_block);
            D.x_smem_elim = xsmem_for(L.op_elim_llt, P);
            D.x_smem_scale = xsmem_for(L.op_scale_llt, P);
            {
                // Gemm ops grouped: forward by neighbour in op order, backward by
                // eliminated cluster in reverse op order.
                std::map<int, std::vector<DGemmOp>> fwd, bwd;
                std::vector<int> fkeys, bkeys;
                for (const GemmOpItem& g : L.op_gemm) {
                    if (!fwd.count(g.nbr)) fkeys.push_back(g.nbr);
                    fwd[g.nbr].push_back({g.self, g.nbr, g.block, g.kind});
                }
                for (auto it = L.op_gemm.rbegin(); it != L.op_gemm.rend(); ++it) {
                    if (!bwd.count(it->self)) bkeys.push_back(it->self);
                    bwd[it->self].push_back({it->self, it->nbr, it->block, it->kind});
                }
                std::vector<DGroup> fg, bg;
                std::vector<DGemmOp> fo, bo;
                for (int k : fkeys) {
                    fg.push_back({k, (int)fo.size(), (int)fwd[k].size()});
                    fo.insert(fo.end(), fwd[k].begin(), fwd[k].end());
                }
                for (int k : bkeys) {
                    bg.push_back({k, (int)bo.size(), (int)bwd[k].size()});
                    bo.insert(bo.end(), bwd[k].begin(), bwd[k].end());
                }
                D.n_gf = (int)fg.size();
                D.n_gb = (int)bg.size();
                D.gf = up(fg);
                D.gb = up(bg);
                D.gfo = up(fo);
                D.gbo = up(bo);
            }
            {
                std::vector<DOrtho> ot;
                int mx = 1;
                for (const auto& wave : L.waves)
                    for (const SparsifyItem& it : wave) {
                        ot.push_back({it.cluster, (long long)it.v_off, (long long)it.tau_off});
                        mx = std::max(mx, P.c_cap[it.cluster]);
                    }
                D.n_ortho = (int)ot.size();
                D.ortho = up(ot);
                D.x_smem_ortho = mx * (int)sizeof(T);
            }
        }
        norms_ = alloc<T>(2 * max_cols);
        jpvt_ = alloc<int>(max_cols);
        ipvt_ = alloc<int>(max_cols);
        colcount_ = alloc<int>(max_items);
        d_xoff_ = up(std::vector<long long>(P.c_xoff.begin(), P.c_xoff.end()));
        xld_ = P.x_len;
        {
            std::vector<long long> slot(perm_h_.size());
            for (int c0 = 0; c0 < nc_; c0++)
                if (P.c_hlevel[c0] == 0)
                    for (int i = 0; i < P.c_cap[c0]; i++) slot[P.c_start[c0] + i] = P.c_xoff[c0] + i;
            d_slot_ = up(slot);
            d_perm_ = up(perm_h_);
        }
        ctx_ = Ctx<T>{arena_, d_blk_, csize_, rows0_, d_cap_, status_};
        SPAND_CUDA(cudaFuncSetAttribute(potrf_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        SPAND_CUDA(cudaFuncSetAttribute(qrcp_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        SPAND_CUDA(cudaFuncSetAttribute(trsv_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        SPAND_CUDA(cudaFuncSetAttribute(ortho_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        caps_h_ = P.c_cap;
    }

    void upload_values(const std::vector<double>& assembled) override {
        if ((int64_t)assembled.size() != P_->assembled_len)
            throw DeviceError{SPAND_ERR_ARG, "assembled values do not match the plan"};
        if (!assembled.empty()) {
            std::vector<T> tmp(assembled.begin(), assembled.end());
            SPAND_CUDA(cudaMemcpyAsync(pristine_, tmp.data(), tmp.size() * sizeof(T), cudaMemcpyHostToDevice, s_));
            SPAND_CUDA(cudaStreamSynchronize(s_));
        }
        factored_ = false;
    }

    void factorize(double tol) override {
        const Plan& P = *P_;
        // inputs: the assembled blocks (device copy) and the initial cluster sizes
        launch("restore", [&] {
            if (P.assembled_len)
                SPAND_CUDA(cudaMemcpyAsync(arena_, pristine_, P.assembled_len * sizeof(T), cudaMemcpyDeviceToDevice, s_));
            if (P.arena_len > P.assembled_len)
                SPAND_CUDA(cudaMemsetAsync(arena_ + P.assembled_len, 0, (P.arena_len - P.assembled_len) * sizeof(T), s_));
            SPAND_CUDA(cudaMemcpyAsync(csize_, d_cap_, nc_ * sizeof(int), cudaMemcpyDeviceToDevice, s_));
            SPAND_CUDA(cudaMemcpyAsync(rows0_, d_cap_, nc_ * sizeof(int), cudaMemcpyDeviceToDevice, s_));
            SPAND_CUDA(cudaMemsetAsync(status_, 0, sizeof(DStatus), s_));
            SPAND_CUDA(cudaMemsetAsync(rank_, 0x7f, nc_ * sizeof(int), s_));
        }, 0);
        for (int l = 0; l < P.nlevels; l++) {
            LevelDev& D = levels_[l];
            if (D.n_elim) {
                launch_potrf(D.elim_pivots, D.elim_clusters, D.n_elim, D.elim_smem);
                launch_trsm(D.elim_trsm0);
                launch_trsm(D.elim_trsm1);
                if (D.n_schur_tiles)
                    launch("schur", [&] {
                        schur_kernel<T><<<D.n_schur_tiles, 256, 0, s_>>>(ctx_, D.schur_targets, d_ups_, D.schur_tiles,
                                                                         D.n_schur_tiles);
                    });
            }
            if (D.scaled && D.n_scale) {
                launch_potrf(D.scale_pivots, D.scale_clusters, D.n_scale, D.scale_smem);
                launch_trsm(D.scale_trsm0);
                launch_trsm(D.scale_trsm1);
            }
            if (D.n_level)
                launch("snapshot", [&] {
                    snapshot_kernel<<<(D.n_level + 255) / 256, 256, 0, s_>>>(csize_, rows0_, D.level_clusters,
                                                                             D.n_level);
                });
            for (WaveDev& W : D.waves) {
                launch("asn_gather", [&] {
                    asn_gather_kernel<T><<<W.n, 256, 0, s_>>>(ctx_, W.items, pieces_, ws_, colcount_);
                });
                launch("qrcp", [&] {
                    qrcp_kernel<T><<<W.n, 512, W.maxcap * sizeof(T), s_>>>(ctx_, W.items, ws_, norms_, jpvt_,
                                                                            colcount_, tauws_, rank_, tol);
                });
                launch("sparsify_scatter", [&] {
                    sparsify_scatter_kernel<T><<<W.n, 256, 0, s_>>>(ctx_, W.items, pieces_, ws_, jpvt_, ipvt_, rank_,
                                                                     vstore_, tauws_, taustore_, colcount_);
                });
            }
            if (D.merged) {
                launch("merge_sizes", [&] {
                    merge_sizes_kernel<<<(D.n_parents + 127) / 128, 128, 0, s_>>>(csize_, rows0_, cpos_, D.parents,
                                                                                    D.n_parents, D.child_ptr,
                                                                                    D.child_idx);
                });
                if (D.n_merge_tiles)
                    launch("merge_copy", [&] {
                        merge_copy_kernel<T><<<D.n_merge_tiles, 256, 0, s_>>>(ctx_, D.merge_items, D.merge_tiles,
                                                                              D.n_merge_tiles, cpos_);
                    });
            }
        }
        SPAND_CUDA(cudaGetLastError());
        DStatus st;
        SPAND_CUDA(cudaMemcpyAsync(&st, status_, sizeof(st), cudaMemcpyDeviceToHost, s_));
        SPAND_CUDA(cudaStreamSynchronize(s_));
        if (st.not_spd)
            throw DeviceError{SPAND_ERR_NOT_SPD, "Error: Non-SPD Pivot (cluster " + std::to_string(st.not_spd - 1) + ")"};
        factored_ = true;
    }

    void solve_device(double* x, int nrhs, int ld) override {
        if (!factored_) throw DeviceError{SPAND_ERR_STATE, "solve before factorize"};
        if (graph_exec_ && graph_x_ == x && graph_nrhs_ == nrhs && graph_ld_ == ld && !prof_.enabled()) {
            SPAND_CUDA(cudaGraphLaunch(graph_exec_, s_));
            launches_ += graph_kernels_;
            return;
        }
        ensure_x(nrhs);
        run_solve(x, nrhs, ld);
    }

    void capture_solve(double* x, int nrhs, int ld) override {
        if (!factored_) throw DeviceError{SPAND_ERR_STATE, "solve before factorize"};
        // the graph reads every size from device memory, so it stays valid across
        // re-factorizations with the same plan
        if (graph_exec_ && graph_x_ == x && graph_nrhs_ == nrhs && graph_ld_ == ld) return;
        ensure_x(nrhs);
        if (graph_exec_) {
            cudaGraphExecDestroy(graph_exec_);
            cudaGraphDestroy(graph_);
            graph_exec_ = nullptr;
            graph_ = nullptr;
        }
        const bool was_on = prof_.enabled();
        prof_.enable(false);
        int64_t before = launches_;
        SPAND_CUDA(cudaStreamBeginCapture(s_, cudaStreamCaptureModeThreadLocal));
        try {
            run_solve(x, nrhs, ld);
        } catch (...) {
            cudaGraph_t g;
            cudaStreamEndCapture(s_, &g);
            if (g) cudaGraphDestroy(g);
            prof_.enable(was_on);
            throw;
        }
        SPAND_CUDA(cudaStreamEndCapture(s_, &graph_));
        SPAND_CUDA(cudaGraphInstantiate(&graph_exec_, graph_, 0));
        prof_.enable(was_on);
        graph_kernels_ = launches_ - before;
        launches_ = before;
        graph_x_ = x;
        graph_nrhs_ = nrhs;
        graph_ld_ = ld;
    }

    void sizes(std::vector<int>& cs, std::vector<int>& r0) override {
        cs.resize(nc_);
        r0.resize(nc_);
        SPAND_CUDA(cudaMemcpyAsync(cs.data(), csize_, nc_ * sizeof(int), cudaMemcpyDeviceToHost, s_));
        SPAND_CUDA(cudaMemcpyAsync(r0.data(), rows0_, nc_ * sizeof(int), cudaMemcpyDeviceToHost, s_));
        SPAND_CUDA(cudaStreamSynchronize(s_));
    }

    void block(int b, std::vector<double>& out) override {
        const PlanBlock& B = P_->blocks[b];
        size_t n = (size_t)B.ld * P_->c_cap[B.colc];
        std::vector<T> tmp(n);
        if (B.flag == BLK_STORED) {
            SPAND_CUDA(cudaMemcpyAsync(tmp.data(), arena_ + B.off, n * sizeof(T), cudaMemcpyDeviceToHost, s_));
            SPAND_CUDA(cudaStreamSynchronize(s_));
        }
        out.assign(tmp.begin(), tmp.end());
    }

    void ortho(int cl, std::vector<double>& v, std::vector<double>& tau) override {
        for (const LevelPlan& L : P_->levels)
            for (const auto& wave : L.waves)
                for (const SparsifyItem& it : wave)
                    if (it.cluster == cl) {
                        size_t n = (size_t)P_->c_cap[cl] * P_->c_cap[cl];
                        std::vector<T> tv(n), tt(P_->c_cap[cl]);
                        SPAND_CUDA(cudaMemcpyAsync(tv.data(), vstore_ + it.v_off, n * sizeof(T), cudaMemcpyDeviceToHost,
                                                   s_));
                        SPAND_CUDA(cudaMemcpyAsync(tt.data(), taustore_ + it.tau_off, tt.size() * sizeof(T),
                                                   cudaMemcpyDeviceToHost, s_));
                        SPAND_CUDA(cudaStreamSynchronize(s_));
                        v.assign(tv.begin(), tv.end());
                        tau.assign(tt.begin(), tt.end());
                        return;
                    }
        v.clear();
        tau.clear();
    }

   private:
    struct TrsmDev {
        DTrsm* items = nullptr;
        DTile* tiles = nullptr;
        int ntiles = 0;
        int side = 0;
    };
    struct WaveDev {
        int n = 0;
        DSpars* items = nullptr;
        int maxcap = 1;
    };
    struct LevelDev {
        int n_elim = 0;
        int* elim_clusters = nullptr;
        int* elim_pivots = nullptr;
        int elim_smem = 0;
        TrsmDev elim_trsm0, elim_trsm1;
        DTarget* schur_targets = nullptr;
        DTile* schur_tiles = nullptr;
        int n_schur_tiles = 0;
        bool scaled = false;
        int n_scale = 0;
        int* scale_clusters = nullptr;
        int* scale_pivots = nullptr;
        int scale_smem = 0;
        TrsmDev scale_trsm0, scale_trsm1;
        int n_level = 0;
        int* level_clusters = nullptr;
        std::vector<WaveDev> waves;
        bool merged = false;
        int n_parents = 0, n_children = 0;
        int *parents = nullptr, *child_ptr = nullptr, *child_idx = nullptr, *child_parent = nullptr;
        DMerge* merge_items = nullptr;
        DTile* merge_tiles = nullptr;
        int n_merge_tiles = 0;
        int n_elim_llt = 0, n_scale_llt = 0;
        int *elim_llt = nullptr, *elim_llt_blk = nullptr, *scale_llt = nullptr, *scale_llt_blk = nullptr;
        int x_smem_elim = 0, x_smem_scale = 0, x_smem_ortho = 0;
        int n_gf = 0, n_gb = 0;
        DGroup *gf = nullptr, *gb = nullptr;
        DGemmOp *gfo = nullptr, *gbo = nullptr;
        int n_ortho = 0;
        DOrtho* ortho = nullptr;
    };

    template <typename V>
    V* alloc(int64_t n) {
        V* p = nullptr;
        SPAND_CUDA(cudaMalloc(&p, std::max<int64_t>(n, 1) * sizeof(V)));
        owned_.push_back(p);
        bytes_ += std::max<int64_t>(n, 1) * sizeof(V);
        return p;
    }
    template <typename V>
    V* up(const std::vector<V>& h) {
        return dev_upload(h, owned_, bytes_, s_);
    }
    // one kernel (or copy) launch: counted, and timed when the profiler is on
    template <typename F>
    void launch(const char* cls, F&& f, int kernels = 1) {
        prof_.begin(s_, cls);
        f();
        prof_.end(s_);
        launches_ += kernels;
    }
    void ensure_x(int nrhs) {
        if (nrhs <= x_nrhs_) return;
        if (xs_) cudaFree(xs_);
        xs_ = nullptr;
        SPAND_CUDA(cudaMalloc(&xs_, (size_t)xld_ * nrhs * sizeof(T)));
        x_nrhs_ = nrhs;
    }
    int smem_for(const std::vector<int>& clusters, const Plan& P) {
        int mx = 0;
        for (int c0 : clusters) mx = std::max(mx, P.c_cap[c0]);
        long long bytes = (long long)mx * mx * sizeof(T);
        return bytes <= 160 * 1024 ? (int)bytes : 0;
    }
    int xsmem_for(const std::vector<int>& clusters, const Plan& P) {
        int mx = 1;
        for (int c0 : clusters) mx = std::max(mx, P.c_cap[c0]);
        if ((int64_t)mx * (int64_t)sizeof(T) > 200 * 1024)
            throw DeviceError{SPAND_ERR_UNSUPPORTED, "cluster too large for the solve kernels"};
        return mx * (int)sizeof(T);
    }
    void build_trsm(const std::vector<TrsmItem>& items, const std::vector<int>& pivots, const std::vector<int>& clusters,
                    const Plan& P, TrsmDev& side0, TrsmDev& side1) {
        std::map<int, int> piv_of;
        for (size_t k = 0; k < clusters.size(); k++) piv_of[clusters[k]] = pivots[k];
        std::vector<DTrsm> it0, it1;
        std::vector<int> ext0, ext1;
        for (const TrsmItem& t : items) {
            const PlanBlock& B = P.blocks[t.block];
            DTrsm d{t.block, piv_of.at(t.cluster), t.cluster, t.side};
            if (t.side == 0) {
                it0.push_back(d);
                ext0.push_back(P.c_cap[B.colc]);
            } else {
                it1.push_back(d);
                ext1.push_back(P.c_cap[B.rowc]);
            }
        }
        auto t0 = tiles_1d(ext0, TRSM_COLS);
        auto t1 = tiles_1d(ext1, TRSM_ROWS);
        side0 = {up(it0), up(t0), (int)t0.size(), 0};
        side1 = {up(it1), up(t1), (int)t1.size(), 1};
    }
    void launch_potrf(int* pivots, int* clusters, int n, int smem) {
        launch("potrf", [&] { potrf_kernel<T><<<n, 256, smem, s_>>>(ctx_, pivots, clusters, n, smem / (int)sizeof(T)); });
    }
    void launch_trsm(const TrsmDev& t) {
        if (!t.ntiles) return;
        launch("trsm", [&] {
            if (t.side == 1) trsm_kernel<T><<<t.ntiles, TRSM_ROWS, 0, s_>>>(ctx_, t.items, t.tiles, t.ntiles);
            else trsm_kernel<T><<<t.ntiles, TRSM_COLS * 32, 0, s_>>>(ctx_, t.items, t.tiles, t.ntiles);
        });
    }

    void run_solve(double* x, int nrhs, int ld) {
        const Plan& P = *P_;
        XCtx<T> X{xs_, (long long)xld_, d_xoff_, nrhs};
        const int n = (int)perm_h_.size();
        const long long tot = (long long)n * nrhs;
        launch("perm", [&] {
            perm_in_kernel<T><<<(unsigned)((tot + 255) / 256), 256, 0, s_>>>(x, ld, X, d_perm_, d_slot_, n);
        });
        for (int l = 0; l < P.nlevels; l++) {
            LevelDev& D = levels_[l];
            if (D.n_elim_llt)
                launch("trsv", [&] {
                    trsv_kernel<T><<<D.n_elim_llt * nrhs, 128, D.x_smem_elim, s_>>>(ctx_, X, D.elim_llt,
                                                                                    D.elim_llt_blk, D.n_elim_llt, 0);
                });
            if (D.n_gf)
                launch("gemm_fwd", [&] { gemm_fwd_kernel<T><<<D.n_gf * nrhs, 128, 0, s_>>>(ctx_, X, D.gf, D.gfo, D.n_gf); });
            if (D.n_scale_llt)
                launch("trsv", [&] {
                    trsv_kernel<T><<<D.n_scale_llt * nrhs, 128, D.x_smem_scale, s_>>>(ctx_, X, D.scale_llt,
                                                                                      D.scale_llt_blk, D.n_scale_llt, 0);
                });
            if (D.n_ortho)
                launch("ortho", [&] {
                    ortho_kernel<T><<<D.n_ortho * nrhs, 128, D.x_smem_ortho, s_>>>(ctx_, X, D.ortho, D.n_ortho, vstore_,
                                                                                   taustore_, 1);
                });
            if (D.merged && D.n_children)
                launch("merge_x", [&] {
                    merge_x_kernel<T><<<D.n_children * nrhs, 128, 0, s_>>>(ctx_, X, D.child_idx, D.child_parent,
                                                                           D.n_children, cpos_, 1);
                });
        }
        for (int l = P.nlevels - 1; l >= 0; l--) {
            LevelDev& D = levels_[l];
            if (D.merged && D.n_children)
                launch("merge_x", [&] {
                    merge_x_kernel<T><<<D.n_children * nrhs, 128, 0, s_>>>(ctx_, X, D.child_idx, D.child_parent,
                                                                           D.n_children, cpos_, 0);
                });
            if (D.n_ortho)
                launch("ortho", [&] {
                    ortho_kernel<T><<<D.n_ortho * nrhs, 128, D.x_smem_ortho, s_>>>(ctx_, X, D.ortho, D.n_ortho, vstore_,
                                                                                   taustore_, 0);
                });
            if (D.n_scale_llt)
                launch("trsv", [&] {
                    trsv_kernel<T><<<D.n_scale_llt * nrhs, 128, D.x_smem_scale, s_>>>(ctx_, X, D.scale_llt,
                                                                                      D.scale_llt_blk, D.n_scale_llt, 1);
                });
            if (D.n_gb)
                launch("gemm_bwd", [&] { gemm_bwd_kernel<T><<<D.n_gb * nrhs, 128, 0, s_>>>(ctx_, X, D.gb, D.gbo, D.n_gb); });
            if (D.n_elim_llt)
                launch("trsv", [&] {
                    trsv_kernel<T><<<D.n_elim_llt * nrhs, 128, D.x_smem_elim, s_>>>(ctx_, X, D.elim_llt,
                                                                                    D.elim_llt_blk, D.n_elim_llt, 1);
                });
        }
        launch("perm", [&] {
            perm_out_kernel<T><<<(unsigned)((tot + 255) / 256), 256, 0, s_>>>(x, ld, X, d_perm_, d_slot_, n);
        });
        SPAND_CUDA(cudaGetLastError());
    }

    cudaStream_t s_;
    std::vector<int> perm_h_;
    std::vector<int> caps_h_;
    const Plan* P_ = nullptr;
    int nc_ = 0;
    std::vector<void*> owned_;
    size_t bytes_ = 0;
    T* arena_ = nullptr;
    T* pristine_ = nullptr;
    DBlock* d_blk_ = nullptr;
    int* d_cap_ = nullptr;
    int *csize_ = nullptr, *rows0_ = nullptr, *rank_ = nullptr, *cpos_ = nullptr;
    DStatus* status_ = nullptr;
    T *vstore_ = nullptr, *taustore_ = nullptr, *tauws_ = nullptr, *ws_ = nullptr, *norms_ = nullptr;
    int *jpvt_ = nullptr, *ipvt_ = nullptr, *colcount_ = nullptr;
    DAsn* pieces_ = nullptr;
    DUpd* d_ups_ = nullptr;
    std::vector<LevelDev> levels_;
    long long* d_xoff_ = nullptr;
    long long* d_slot_ = nullptr;
    int* d_perm_ = nullptr;
    int64_t xld_ = 0;
    T* xs_ = nullptr;
    int x_nrhs_ = 0;
    Ctx<T> ctx_{};
    bool factored_ = false;
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t graph_exec_ = nullptr;
    int64_t graph_kernels_ = 0;
    double* graph_x_ = nullptr;
    int graph_nrhs_ = 0, graph_ld_ = 0;
};

std::unique_ptr<DeviceFactorBase> make_device_factor(bool fp32, cudaStream_t stream, const std::vector<int>& perm) {
    if (fp32) return std::unique_ptr<DeviceFactorBase>(new DeviceFactor<float>(stream, perm));
    return std::unique_ptr<DeviceFactorBase>(new DeviceFactor<double>(stream, perm));
}

void device_spmv(const DeviceCsr& A, const double* x, double* y, cudaStream_t s) {
    spmv_kernel<<<(A.n + 255) / 256, 256, 0, s>>>(A.n, A.rowptr, A.colind, A.val, x, y);
}

// Workspace of the device CG, kept across calls for one matrix size.
struct PcgWork {
    int n = 0;
    double *r = nullptr, *p = nullptr, *z = nullptr, *tmp = nullptr, *partial = nullptr, *sc = nullptr;
    double* h_sc = nullptr;
    ~PcgWork() { release(); }
    void release() {
        cudaFree(r); cudaFree(p); cudaFree(z); cudaFree(tmp); cudaFree(partial); cudaFree(sc);
        if (h_sc) cudaFreeHost(h_sc);
        r = p = z = tmp = partial = sc = h_sc = nullptr;
        n = 0;
    }
    void ensure(int nn) {
        if (nn == n) return;
        release();
        SPAND_CUDA(cudaMalloc(&r, nn * sizeof(double)));
        SPAND_CUDA(cudaMalloc(&p, nn * sizeof(double)));
        SPAND_CUDA(cudaMalloc(&z, nn * sizeof(double)));
        SPAND_CUDA(cudaMalloc(&tmp, nn * sizeof(double)));
        SPAND_CUDA(cudaMalloc(&partial, RED_BLOCKS * sizeof(double)));
        SPAND_CUDA(cudaMalloc(&sc, 8 * sizeof(double)));
        SPAND_CUDA(cudaMallocHost(&h_sc, 8 * sizeof(double)));
        n = nn;
    }
};

static thread_local PcgWork g_pcg;

// Preconditioned CG (is.cpp:39-121) with all vectors and scalars on the device; one
// scalar read back per iteration for the stopping test.
PcgResult device_pcg(DeviceFactorBase& M, const DeviceCsr& A, const double* b, double* x, int maxit, double tol,
                     bool use_graph) {
    cudaStream_t s = M.stream();
    KernelProfiler& prof = M.profiler();
    const int n = A.n;
    PcgResult res;
    g_pcg.ensure(n);
    double *r = g_pcg.r, *p = g_pcg.p, *z = g_pcg.z, *tmp = g_pcg.tmp, *partial = g_pcg.partial, *sc = g_pcg.sc;
    double* h_sc = g_pcg.h_sc;
    auto L = [&](const char* cls, auto&& f, int k = 1) {
        prof.begin(s, cls);
        f();
        prof.end(s);
        M.add_launches(k);
    };
    const unsigned gb = (unsigned)((n + 255) / 256);
    auto dot = [&](const double* a, const double* bb, int slot) {
        L("dot", [&] {
            dot_partial_kernel<<<RED_BLOCKS, RED_THREADS, 0, s>>>(n, a, bb, partial);
            dot_final_kernel<<<1, RED_THREADS, 0, s>>>(partial, RED_BLOCKS, sc + slot);
        }, 2);
    };
    auto spmv = [&](const double* in, double* out) {
        L("spmv", [&] { spmv_kernel<<<gb, 256, 0, s>>>(n, A.rowptr, A.colind, A.val, in, out); });
    };
    spmv(x, tmp);
    L("axpy", [&] { sub_kernel<<<gb, 256, 0, s>>>(n, b, tmp, r); });
    dot(b, b, 4);
    dot(r, r, 2);
    SPAND_CUDA(cudaMemcpyAsync(h_sc, sc, 8 * sizeof(double), cudaMemcpyDeviceToHost, s));
    SPAND_CUDA(cudaStreamSynchronize(s));
    const double rhsNorm2 = h_sc[4];
    if (rhsNorm2 == 0) {
        SPAND_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), s));
        SPAND_CUDA(cudaStreamSynchronize(s));
        return res;
    }
    const double threshold = tol * tol * rhsNorm2;
    double resNorm2 = h_sc[2];
    res.relres = std::sqrt(resNorm2 / rhsNorm2);
    if (resNorm2 < threshold) return res;
    SPAND_CUDA(cudaMemcpyAsync(p, r, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    M.solve_device(p, 1, n);
    dot(r, p, 0);
    if (use_graph) M.capture_solve(z, 1, n);
    int i = 0;
    while (i < maxit) {
        spmv(p, tmp);
        dot(p, tmp, 1);
        L("axpy", [&] { cg_update_xr_kernel<<<gb, 256, 0, s>>>(n, x, r, p, tmp, sc); });
        dot(r, r, 2);
        SPAND_CUDA(cudaMemcpyAsync(h_sc + 2, sc + 2, sizeof(double), cudaMemcpyDeviceToHost, s));
        SPAND_CUDA(cudaStreamSynchronize(s));
        resNorm2 = h_sc[2];
        if (resNorm2 < threshold) break;
        SPAND_CUDA(cudaMemcpyAsync(z, r, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        M.solve_device(z, 1, n);
        L("axpy", [&] { copy_scalar_kernel<<<1, 1, 0, s>>>(sc, 3, 0); });
        dot(r, z, 0);
        L("axpy", [&] { cg_update_p_kernel<<<gb, 256, 0, s>>>(n, p, z, sc); });
        i++;
    }
    SPAND_CUDA(cudaGetLastError());
    res.iterations = i + 1;
    res.relres = std::sqrt(resNorm2 / rhsNorm2);
    return res;
}

}  // namespace spand

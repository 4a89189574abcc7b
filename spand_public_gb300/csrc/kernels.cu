// CUDA kernels and the device driver of the GB300 spaND factorization and solve.
//
// Every kernel reads cluster sizes from device memory (csize: current size, rows0: size
// when the cluster's hierarchy level started).  Work lists are uploaded once from the
// symbolic plan; grids are sized from capacities and surplus blocks exit early.
// Citations are path:line into leopoldcambier/spaND_public.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <climits>
#include <cstring>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "device.h"
#include "kcommon.cuh"
#include "preserve.cuh"
#include "qrcp.cuh"

namespace spand {

// Inverse of a lower Cholesky factor, written transposed into the strictly upper triangle
// of the same block: after the call, for i > j, A[j + i*ld] = (L^{-1})[i][j]; the diagonal
// of L^{-1} is 1/L[i][i] and is not stored.  Right-looking forward substitution on all
// columns of the identity at once (n steps, two barriers each).
template <typename T>
__device__ void trtri_to_upper(T* A, int ld, int n) {
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
        int j = idx % n, i = idx / n;
        if (i > j) A[j + (size_t)i * ld] = T(0);
    }
    __syncthreads();
    for (int k = 0; k < n; k++) {
        const T dinv = T(1) / A[k + (size_t)k * ld];
        for (int j = threadIdx.x; j < k; j += blockDim.x) A[j + (size_t)k * ld] *= dinv;
        __syncthreads();
        // R[i, j] -= L[i, k] * Y[k, j] for i > k, j <= k
        const int m = n - k - 1, w = k + 1;
        for (int idx = threadIdx.x; idx < m * w; idx += blockDim.x) {
            const int j = idx % w, i = k + 1 + idx / w;
            const T ykj = (j == k) ? dinv : A[j + (size_t)k * ld];
            A[j + (size_t)i * ld] -= A[i + (size_t)k * ld] * ykj;
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------------------------
// Cholesky of pivot blocks in place in global memory, blocked left-looking with 32-column
// panels (dpotrf 'L', tree.cpp:582-593): the path of pivots too large for shared memory.
// Per panel: (1) update by the factored columns, (2) the 32x32 diagonal block by one warp
// with shuffles, (3) the rows below by a triangular solve, one row per thread.  Three
// barriers per panel.  (Pivots that fit are factored and inverted by chol_inv_tiled.)
// ------------------------------------------------------------------------------------
constexpr int PNB = 32;

template <typename T>
__device__ bool chol_blocked(T* A, int ld, int n, int* bad) {
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5, nty = blockDim.x >> 5;
    for (int jb = 0; jb < n; jb += PNB) {
        const int w = min(PNB, n - jb);
        if (jb > 0) {
            for (int jj = ty; jj < w; jj += nty) {
                const int j = jb + jj;
                for (int i = j + tx; i < n; i += 32) {
                    T s0 = 0, s1 = 0, s2 = 0, s3 = 0;
                    int k = 0;
                    for (; k + 3 < jb; k += 4) {
                        s0 += A[i + (size_t)k * ld] * A[j + (size_t)k * ld];
                        s1 += A[i + (size_t)(k + 1) * ld] * A[j + (size_t)(k + 1) * ld];
                        s2 += A[i + (size_t)(k + 2) * ld] * A[j + (size_t)(k + 2) * ld];
                        s3 += A[i + (size_t)(k + 3) * ld] * A[j + (size_t)(k + 3) * ld];
                    }
                    for (; k < jb; k++) s0 += A[i + (size_t)k * ld] * A[j + (size_t)k * ld];
                    A[i + (size_t)j * ld] -= (s0 + s1) + (s2 + s3);
                }
            }
            __syncthreads();
        }
        if (ty == 0) {
            int fail = 0;
            for (int j = 0; j < w; j++) {
                T* cj = A + (size_t)(jb + j) * ld + jb;
                T d = 0;
                if (tx == j) {
                    d = cj[j];
                    if (!(d > T(0))) {
                        fail = 1;
                        d = T(1);
                    } else {
                        d = dsqrt(d);
                    }
                    cj[j] = d;
                }
                d = __shfl_sync(0xffffffffu, d, j);
                fail = __shfl_sync(0xffffffffu, fail, j);
                if (fail) break;
                if (tx > j && tx < w) cj[tx] /= d;
                __syncwarp();
                if (tx > j && tx < w) {
                    const T lij = cj[tx];
                    for (int kk = j + 1; kk <= tx; kk++) A[(jb + tx) + (size_t)(jb + kk) * ld] -= lij * cj[kk];
                }
                __syncwarp();
            }
            if (tx == 0 && fail) *bad = 1;
        }
        __syncthreads();
        if (*bad) return false;
        // rows below the diagonal block: x_j = (a_j - sum_{l<j} x_l L[jb+j][jb+l]) / L[jb+j][jb+j]
        for (int i = jb + w + threadIdx.x; i < n; i += blockDim.x) {
            for (int j = 0; j < w; j++) {
                T x = A[i + (size_t)(jb + j) * ld];
                for (int l = 0; l < j; l++) x -= A[i + (size_t)(jb + l) * ld] * A[(jb + j) + (size_t)(jb + l) * ld];
                A[i + (size_t)(jb + j) * ld] = x / A[(jb + j) + (size_t)(jb + j) * ld];
            }
        }
        __syncthreads();
    }
    return true;
}

// The 32x32 diagonal block of a panel (rows and columns jb..jb+w-1 of a block held in shared
// memory with leading dimension ld), by the first warp.  Cholesky in registers, lane i
// holding row i (a[k] = A[i][k], k <= i), right-looking with the columns broadcast by
// shuffles; each step scales by r = 1/sqrt(pivot) (L[j][j] = pivot * r, the column below
// times r), and lane j keeps r = 1/L[j][j].  Then the inverse D, column c = lane in registers,
// by forward substitution, D[r][c] = (delta_rc - sum_{l<r} L[r][l] D[l][c]) / L[r][r], each
// sum in four interleaved partial sums (a quarter of the dependent chain; the L[r][l] are
// broadcast loads) and the division a product with 1/L[r][r].  D goes transposed into the block's strictly upper slots (A[(jb+c) + (jb+r)*ld] = D[r][c],
// r > c) and row-major into Dpad (zero above the diagonal and outside w) for the rows
// below.  Sets *bad on a non-positive pivot.
template <typename T>
__device__ void chol_diag32(T* A, int ld, int jb, int w, T* Dpad, int* bad) {
    const int lane = threadIdx.x & 31;
    T a[PNB];
#pragma unroll
    for (int k = 0; k < PNB; k++) a[k] = (k <= lane && lane < w) ? A[(jb + lane) + (jb + k) * ld] : T(0);
    int fail = 0;
    T rl = T(1);  // 1 / L[lane][lane]
#pragma unroll
    for (int j = 0; j < PNB; j++) {
        if (j < w) {
            const T t = __shfl_sync(0xffffffffu, a[j], j);
            T r = T(1);
            if (!(t > T(0))) fail = 1;
            else r = rsqrt_t(t);
            if (lane == j) {
                a[j] = t * r;
                rl = r;
            } else if (lane > j) {
                a[j] *= r;
            }
            const T lij = a[j];
#pragma unroll
            for (int k = j + 1; k < PNB; k++) {
                const T lkj = __shfl_sync(0xffffffffu, a[j], k);
                if (lane > j && k <= lane) a[k] -= lij * lkj;
            }
        }
    }
    if (lane < w)
#pragma unroll
        for (int k = 0; k < PNB; k++)
            if (k <= lane) A[(jb + lane) + (jb + k) * ld] = a[k];
    __syncwarp();
    if (lane == 0 && fail) *bad = 1;
    if (fail) return;
    T d[PNB];
#pragma unroll
    for (int r = 0; r < PNB; r++) {
        d[r] = T(0);
        if (r < w) {
            T s0 = r == lane ? T(1) : T(0), s1 = T(0), s2 = T(0), s3 = T(0);
#pragma unroll
            for (int l = 0; l < r; l += 4) {
                s0 -= A[(jb + r) + (jb + l) * ld] * d[l];
                if (l + 1 < r) s1 -= A[(jb + r) + (jb + l + 1) * ld] * d[l + 1];
                if (l + 2 < r) s2 -= A[(jb + r) + (jb + l + 2) * ld] * d[l + 2];
                if (l + 3 < r) s3 -= A[(jb + r) + (jb + l + 3) * ld] * d[l + 3];
            }
            d[r] = ((s0 + s1) + (s2 + s3)) * __shfl_sync(0xffffffffu, rl, r);
        }
    }
#pragma unroll
    for (int r = 0; r < PNB; r++) {
        if (r < w && r > lane) A[(jb + lane) + (jb + r) * ld] = d[r];
        Dpad[r * (PNB + 1) + lane] = d[r];
    }
}

// Cholesky and inverse of a pivot block held in shared memory (ld = n, lower triangle
// in, L in the lower triangle and L^{-1} transposed in the strictly upper triangle out;
// the diagonal of L^{-1}, 1 / L_ii, is not stored).  32-column panels: (1) update of the
// panel by the factored columns (left-looking), (2) the 32x32 diagonal block and its
// inverse D (chol_diag32), (3) rows below: row x D^T, a warp per row.  Then L^{-1} block row
// by block row: L^{-1}[I][J] = -D_I sum_{J <= K < I} L[I][K] L^{-1}[K][J], the sum written
// into the block's upper-triangle slots first and multiplied by D_I per column.  256
// threads, one element per thread in the products (kept as the comparison path of
// chol_inv_tiled).
template <typename T>
__device__ bool chol_inv_smem(T* A, int n, int* bad, T* Dpad) {
    const int tid = threadIdx.x, lane = tid & 31, w8 = tid >> 5;
    constexpr int NWARP = 8;
    const int nb = (n + PNB - 1) / PNB;
    for (int pb = 0; pb < nb; pb++) {
        const int jb = pb * PNB, w = min(PNB, n - jb);
        // (1) left-looking update of the panel
        if (jb > 0) {
            for (int jj = w8; jj < w; jj += NWARP) {
                const int j = jb + jj;
                for (int i = j + lane; i < n; i += 32) {
                    T s0 = 0, s1 = 0, s2 = 0, s3 = 0;
                    int k = 0;
                    for (; k + 3 < jb; k += 4) {
                        s0 += A[i + k * n] * A[j + k * n];
                        s1 += A[i + (k + 1) * n] * A[j + (k + 1) * n];
                        s2 += A[i + (k + 2) * n] * A[j + (k + 2) * n];
                        s3 += A[i + (k + 3) * n] * A[j + (k + 3) * n];
                    }
                    for (; k < jb; k++) s0 += A[i + k * n] * A[j + k * n];
                    A[i + j * n] -= (s0 + s1) + (s2 + s3);
                }
            }
            __syncthreads();
        }
        // (2) diagonal block and its inverse (upper-triangle slots of the block)
        if (tid < 32) chol_diag32(A, n, jb, w, Dpad, bad);
        __syncthreads();
        if (*bad) return false;
        // (3) rows below: L[i][jb+j] = sum_{l <= j} A[i][jb+l] D[j][l]
        for (int i = jb + w + w8; i < n; i += NWARP) {
            T out = 0;
            if (lane < w)
                for (int l = 0; l <= lane; l++) out += A[i + (jb + l) * n] * Dpad[lane * (PNB + 1) + l];
            __syncwarp();
            if (lane < w) A[i + (jb + lane) * n] = out;
        }
        __syncthreads();
    }
    // off-diagonal blocks of L^{-1}, block row by block row
    for (int ib = 1; ib < nb; ib++) {
        const int i0 = ib * PNB, h = min(PNB, n - i0);
        // E[i][j] = sum_{j <= m < i0} L[i][m] Linv[m][j] for rows i in the block, j < i0
        for (int idx = tid; idx < h * i0; idx += blockDim.x) {
            const int ii = idx % h, j = idx / h;
            const int i = i0 + ii;
            T sum = A[i + j * n] / A[j + j * n];  // m = j: Linv[j][j] = 1 / L[j][j]
            for (int m = j + 1; m < i0; m++) sum += A[i + m * n] * A[j + m * n];
            A[j + i * n] = sum;
        }
        __syncthreads();
        // Linv[i][j] = -sum_{l <= i} D[i][l] E[l][j] (block rows, D = diagonal block inverse)
        for (int j = tid; j < i0; j += blockDim.x) {
            T e[PNB];
#pragma unroll
            for (int l = 0; l < PNB; l++) e[l] = l < h ? A[j + (i0 + l) * n] : T(0);
#pragma unroll
            for (int ii = PNB - 1; ii >= 0; ii--) {
                if (ii < h) {
                    T sum = e[ii] / A[(i0 + ii) + (i0 + ii) * n];
#pragma unroll
                    for (int l = 0; l < ii; l++) sum += A[(i0 + l) + (i0 + ii) * n] * e[l];
                    A[j + (i0 + ii) * n] = -sum;
                }
            }
        }
        __syncthreads();
    }
    return true;
}

// Elements of a pivot block of n rows held in shared memory by chol_inv_tiled: leading
// dimension n rounded up to a multiple of four, so that four consecutive rows starting at a
// multiple of four are one 16-byte load
__host__ __device__ inline int potrf_ld(int n) { return (n + 3) & ~3; }
constexpr int POTRF_SMEM_MAX = 216 * 1024;  // dynamic shared memory of potrf3_kernel at most
// above this, a level's one-CTA Cholesky is launched per size class (three CTAs of 256
// threads per SM fit beside it)
constexpr int POTRF_MID_SMEM = 68 * 1024;
__host__ __device__ inline long long potrf_held(int n) { return (long long)potrf_ld(n) * n; }

// The same factorization and inverse, same layout (leading dimension ld = potrf_ld(n)) and
// results up to rounding, with every product of the panels on register tiles: a thread
// holds 4 rows x 4 columns of the output (8 column groups x 32 row groups over the 256
// threads) and reads each group of four rows or columns as one 16-byte load, so two loads
// feed sixteen multiply-adds and sixteen independent sums are in flight.  (1) the panel's
// left-looking update, rows jb..n-1 in passes of 128; (3) the rows below times D^T; then per
// block row I of L^{-1}: (a) E = L[I][0:i0] L^{-1}[0:i0][0:i0] on tiles of E into the block's
// upper slots, a thread taking column group g and, past 32 groups, its mirror (the sums
// shorten with the column, so the pair's work is even); (b) L^{-1}[I][0:i0] = -D_I E on
// tiles, read into registers, a barrier, then written over E (the tiles of one pass cover
// disjoint column groups from the next pass's).  Rows between n and ld are read as padding
// and never written back.
template <typename T>
__device__ bool chol_inv_tiled(T* A, int n, int ld, int* bad, T* Dpad) {
    const int tid = threadIdx.x;
    const int cq = tid & 7, rq = tid >> 3;  // the thread's 4-column group and 4-row group
    const int c0 = 4 * cq;
    const int nb = (n + PNB - 1) / PNB;
    for (int pb = 0; pb < nb; pb++) {
        const int jb = pb * PNB, w = min(PNB, n - jb);
        // (1) A[i][jb+jj] -= sum_{k < jb} L[i][k] L[jb+jj][k], i >= jb + jj
        if (jb > 0) {
            for (int r0 = jb + 4 * rq; r0 < n; r0 += 128) {
                if (r0 + 3 < jb + c0 || c0 >= w) continue;  // above the diagonal or right of the panel
                T acc[4][4];
#pragma unroll
                for (int u = 0; u < 4; u++)
#pragma unroll
                    for (int v = 0; v < 4; v++) acc[u][v] = T(0);
                const T* pa = A + r0;
                const T* pbk = A + jb + c0;
#pragma unroll 2
                for (int k = 0; k < jb; k++) {
                    T a[4], b[4];
                    lds4(pa + k * ld, a);
                    lds4(pbk + k * ld, b);
#pragma unroll
                    for (int u = 0; u < 4; u++)
#pragma unroll
                        for (int v = 0; v < 4; v++) acc[u][v] += a[u] * b[v];
                }
#pragma unroll
                for (int u = 0; u < 4; u++)
#pragma unroll
                    for (int v = 0; v < 4; v++) {
                        const int i = r0 + u, jj = c0 + v;
                        if (i < n && jj < w && i >= jb + jj) A[i + (jb + jj) * ld] -= acc[u][v];
                    }
            }
            __syncthreads();
        }
        // (2) diagonal block and its inverse
        if (tid < 32) chol_diag32(A, ld, jb, w, Dpad, bad);
        __syncthreads();
        if (*bad) return false;
        // (3) rows below: L[i][jb+c] = sum_{l <= c} A[i][jb+l] D[c][l] (Dpad zero above its
        // diagonal); the eight threads of a row group share a warp, which has read all its rows
        // before any of them is written
        for (int base = jb + w; base < n; base += 128) {
            const int r0 = base + 4 * rq;
            const bool act = r0 < n && c0 < w;
            T acc[4][4];
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int v = 0; v < 4; v++) acc[u][v] = T(0);
            if (act) {
                const int lmax = min(c0 + 3, w - 1);
                for (int l = 0; l <= lmax; l++) {
                    T a[4], d[4];
                    lds4(A + r0 + (jb + l) * ld, a);
#pragma unroll
                    for (int v = 0; v < 4; v++) d[v] = Dpad[(c0 + v) * (PNB + 1) + l];
#pragma unroll
                    for (int u = 0; u < 4; u++)
#pragma unroll
                        for (int v = 0; v < 4; v++) acc[u][v] += a[u] * d[v];
                }
            }
            __syncwarp();
            if (act)
#pragma unroll
                for (int u = 0; u < 4; u++)
#pragma unroll
                    for (int v = 0; v < 4; v++)
                        if (r0 + u < n && c0 + v < w) A[(r0 + u) + (jb + c0 + v) * ld] = acc[u][v];
        }
        __syncthreads();
    }
    // off-diagonal blocks of L^{-1}, block row by block row; a tile is a row group q = 4 *
    // (0..7) (rows i0+q..+3 of the block) and a column group j0 = 4 * g (columns j0..j0+3 < i0)
    for (int ib = 1; ib < nb; ib++) {
        const int i0 = ib * PNB, h = min(PNB, n - i0);
        const int ng = i0 / 4;  // column groups
        const int q = 4 * (tid & 7);
        // (a) E[ii][j] = sum_{j <= m < i0} L[i0+ii][m] Linv[m][j] -> A[j + (i0+ii)*ld]
        if (q < h) {
            for (int pass = 0; pass < 2; pass++) {
                const int g = pass == 0 ? (tid >> 3) : ng - 1 - (tid >> 3);
                if (g >= ng || (pass == 1 && g < 32)) break;
                const int j0 = 4 * g;
                T acc[4][4];
#pragma unroll
                for (int u = 0; u < 4; u++)
#pragma unroll
                    for (int v = 0; v < 4; v++) acc[u][v] = T(0);
                // m = j0..j0+3: Linv[m][j0+v] is 0 above its diagonal and 1 / L[m][m] on it
#pragma unroll
                for (int mm = 0; mm < 4; mm++) {
                    const int m = j0 + mm;
                    const T rd = T(1) / A[m + m * ld];
                    T a[4], b[4];
                    lds4(A + i0 + q + m * ld, a);
#pragma unroll
                    for (int v = 0; v < 4; v++) b[v] = mm < v ? T(0) : (mm == v ? rd : A[(j0 + v) + m * ld]);
#pragma unroll
                    for (int u = 0; u < 4; u++)
#pragma unroll
                        for (int v = 0; v < 4; v++) acc[u][v] += a[u] * b[v];
                }
#pragma unroll 2
                for (int m = j0 + 4; m < i0; m++) {
                    T a[4], b[4];
                    lds4(A + i0 + q + m * ld, a);
                    lds4(A + j0 + m * ld, b);
#pragma unroll
                    for (int u = 0; u < 4; u++)
#pragma unroll
                        for (int v = 0; v < 4; v++) acc[u][v] += a[u] * b[v];
                }
#pragma unroll
                for (int u = 0; u < 4; u++)
                    if (q + u < h)
#pragma unroll
                        for (int v = 0; v < 4; v++) A[(j0 + v) + (i0 + q + u) * ld] = acc[u][v];
            }
        }
        __syncthreads();
        // (b) Linv[i0+ii][j] = -(E[ii][j] / L[i0+ii][i0+ii] + sum_{l < ii} D[ii][l] E[l][j]),
        // D[ii][l] = A[(i0+l) + (i0+ii)*ld]; column group g = t >> 3 of tile t
        const int ntile = 8 * ng;
        for (int t0 = 0; t0 < ntile; t0 += blockDim.x) {
            const int t = t0 + tid;
            const bool act = t < ntile && q < h;
            const int j0 = 4 * (t >> 3);
            T o[4][4];
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int v = 0; v < 4; v++) o[u][v] = T(0);
            if (act) {
                int co[4];
#pragma unroll
                for (int u = 0; u < 4; u++) co[u] = min(i0 + q + u, n - 1) * ld;
                for (int l = 0; l < q; l++) {  // below every row of the group: D[q+u][l] stored
                    T d[4], e[4];
#pragma unroll
                    for (int u = 0; u < 4; u++) d[u] = A[(i0 + l) + co[u]];
                    lds4(A + j0 + (i0 + l) * ld, e);
#pragma unroll
                    for (int u = 0; u < 4; u++)
#pragma unroll
                        for (int v = 0; v < 4; v++) o[u][v] += d[u] * e[v];
                }
#pragma unroll
                for (int ll = 0; ll < 4; ll++) {  // l = q..q+3: the group's own triangle
                    const int l = q + ll;
                    if (l < h) {
                        T d[4], e[4];
#pragma unroll
                        for (int u = 0; u < 4; u++)
                            d[u] = ll < u ? A[(i0 + l) + co[u]] : (ll == u ? T(1) / A[(i0 + l) + (i0 + l) * ld] : T(0));
                        lds4(A + j0 + (i0 + l) * ld, e);
#pragma unroll
                        for (int u = 0; u < 4; u++)
#pragma unroll
                            for (int v = 0; v < 4; v++) o[u][v] += d[u] * e[v];
                    }
                }
            }
            __syncthreads();
            if (act)
#pragma unroll
                for (int u = 0; u < 4; u++)
                    if (q + u < h)
#pragma unroll
                        for (int v = 0; v < 4; v++) A[(j0 + v) + (i0 + q + u) * ld] = -o[u][v];
        }
        __syncthreads();
    }
    return true;
}

template <typename T>
// FP32: registers capped for three CTAs per SM (24 bytes of spills); FP64 keeps two
// (its register-resident panels would spill hundreds of bytes)
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 2) potrf3_kernel(Ctx<T> c, const int* __restrict__ pivots,
                                                     const int* __restrict__ clusters, int count, int smem_elems,
                                                     int strip_max_n, const int* __restrict__ only,
                                                     int small_cap, int tiled, int n_lo, int n_hi) {
    pdl_wait_and_release();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sm = reinterpret_cast<T*>(smem_raw);
    const int item = blockIdx.x;
    if (item >= count || (only && !only[item])) return;
    __shared__ int failed;
    __shared__ int bad;
    if (threadIdx.x == 0) {
        failed = *(volatile int*)&c.status->not_spd;
        bad = 0;
    }
    __syncthreads();
    if (failed) return;
    const int cl = clusters[item];
    const int n = c.csize[cl];
    if (n == 0 || c.cap[cl] <= small_cap) return;  // small pivots: potrf_small_kernel
    if (n <= n_lo || n > n_hi) return;              // the other size class's launch
    T* G = bptr(c, pivots[item]);
    const int gld = c.blk[pivots[item]].ld;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5, nty = blockDim.x >> 5;
    if (potrf_held(n) <= smem_elems) {
        const int ld = tiled ? potrf_ld(n) : n;
        // the lower triangle, two columns per warp at a time with up to sixteen loads in flight
        // per lane before their stores (a load behind a shared-memory store it may alias would
        // otherwise wait out the previous load: one HBM latency per element a lane copies)
        for (int j0 = ty; j0 < n; j0 += 2 * nty) {
            for (int r = 0; r < n - j0; r += 256) {
                T v[2][8];
#pragma unroll
                for (int cc = 0; cc < 2; cc++) {
                    const int j = j0 + cc * nty;
#pragma unroll
                    for (int m = 0; m < 8; m++) {
                        const int i = j + r + tx + 32 * m;
                        v[cc][m] = (j < n && i < n) ? G[i + (size_t)j * gld] : T(0);
                    }
                }
#pragma unroll
                for (int cc = 0; cc < 2; cc++) {
                    const int j = j0 + cc * nty;
#pragma unroll
                    for (int m = 0; m < 8; m++) {
                        const int i = j + r + tx + 32 * m;
                        if (j < n && i < n) sm[i + j * ld] = v[cc][m];
                    }
                }
            }
        }
        __syncthreads();
        // factor and inverse together; the whole block (L below, L^{-1} transposed above) back
        __shared__ T Dpad[PNB * (PNB + 1)];  // inverse of the current diagonal block, padded rows
        if (tiled ? chol_inv_tiled(sm, n, ld, &bad, Dpad) : chol_inv_smem(sm, n, &bad, Dpad)) {
            for (int j = ty; j < n; j += nty)
                for (int i = tx; i < n; i += 32) G[i + (size_t)j * gld] = sm[i + j * ld];
        }
    } else {
        chol_blocked(G, gld, n, &bad);
        __syncthreads();
        // pivots the strip-wise inverse kernel does not take get their inverse here
        if (!bad && n > strip_max_n) trtri_to_upper(G, gld, n);
    }
    if (bad && threadIdx.x == 0) atomicCAS(&c.status->not_spd, 0, cl + 1);
}

// Pivots of at most 32 rows, one warp each (eight per CTA), in registers: lane i holds row
// i of the block (a[k] = A[i][k], k <= i); right-looking Cholesky with the columns
// broadcast by shuffles (the same operations per element, in the same order, as
// chol_inv_smem's diagonal block), then column c = lane of L^{-1} by forward substitution
// with L's rows broadcast by shuffles.  Out: L in the lower triangle, L^{-1} transposed in
// the strictly upper one (the layout of potrf3_kernel).  The thousands of small pivots of
// the lowest levels otherwise take a 256-thread CTA each, two per SM (the large kernel's
// registers), for a few hundred FMAs.
constexpr int PS_WARPS = 8;
template <typename T>
__global__ void __launch_bounds__(32 * PS_WARPS) potrf_small_kernel(Ctx<T> c, const int* __restrict__ pivots,
                                                                   const int* __restrict__ clusters, int count) {
    pdl_wait_and_release();
    const int lane = threadIdx.x & 31;
    const int k = blockIdx.x * PS_WARPS + (threadIdx.x >> 5);
    if (k >= count) return;
    if (*(volatile int*)&c.status->not_spd) return;
    const int item = k;
    const int cl = clusters[item];
    const int n = c.csize[cl];
    if (n == 0 || n > 32) return;
    T* G = bptr(c, pivots[item]);
    const int ld = c.blk[pivots[item]].ld;
    T a[32];
#pragma unroll
    for (int q = 0; q < 32; q++) a[q] = (q <= lane && lane < n) ? G[lane + (size_t)q * ld] : T(0);
    int fail = 0;
#pragma unroll
    for (int j = 0; j < 32; j++) {
        if (j < n) {
            T d = __shfl_sync(0xffffffffu, a[j], j);
            if (!(d > T(0))) {
                fail = 1;
                d = T(1);
            } else {
                d = dsqrt(d);
            }
            if (lane == j) a[j] = d;
            else if (lane > j) a[j] /= d;
            const T lij = a[j];
#pragma unroll
            for (int q = j + 1; q < 32; q++) {
                const T lqj = __shfl_sync(0xffffffffu, a[j], q);
                if (lane > j && q <= lane) a[q] -= lij * lqj;
            }
        }
    }
    if (__any_sync(0xffffffffu, fail)) {
        if (lane == 0) atomicCAS(&c.status->not_spd, 0, cl + 1);
        return;
    }
    // D = L^{-1}, column c = lane: D[r][c] = (delta_rc - sum_{c <= l < r} L[r][l] D[l][c]) / L[r][r]
    T dcol[32];
#pragma unroll
    for (int r = 0; r < 32; r++) {
        T acc = r == lane ? T(1) : T(0);
#pragma unroll
        for (int l = 0; l < r; l++) acc -= __shfl_sync(0xffffffffu, a[l], r) * dcol[l];
        const T lrr = __shfl_sync(0xffffffffu, a[r], r);
        dcol[r] = (r >= lane && r < n) ? acc / lrr : T(0);
    }
    if (lane < n) {
#pragma unroll
        for (int q = 0; q < 32; q++)
            if (q <= lane) G[lane + (size_t)q * ld] = a[q];  // L, row lane
#pragma unroll
        for (int r = 0; r < 32; r++)
            if (r > lane && r < n) G[lane + (size_t)r * ld] = dcol[r];  // L^{-1}[r][lane] at (lane, r)
    }
}

// Cholesky factorization of pivot blocks too large for one CTA's shared memory, in the
// shared memory of a thread-block cluster of CS CTAs (LLT pivots, src/tree.cpp:587-590).
// The lower triangle is cut into 32-column panels; panel p (rows [32p, n)) lives in CTA
// p mod CS.  Per panel: the owner factors the 32x32 diagonal block in one warp's registers
// (a row per lane, columns broadcast by shuffles), inverts it (a column of the inverse per
// lane) and forms the rows below as products with that inverse, four rows per warp at a
// time (no sequential substitution over the columns); one cluster barrier; every CTA
// copies the panel's trailing rows through distributed shared memory and applies them to
// its own later panels (4x4 register tiles).  A non-SPD diagonal stops every CTA after
// the barrier.  Pivots whose panels exceed smem_bytes set fallback[item] (the
// single-CTA kernel then factors them from global memory).
constexpr int PC_THREADS = 256;

// shared memory of CTA r: its panels of an n x n pivot plus one staged panel
__host__ __device__ inline long long pc_need(int n, int cs, int r, int elem) {
    long long e = 0;
    const int np = (n + 31) / 32;
    for (int p = r; p < np; p += cs) e += (long long)(n - 32 * p) * 32;
    return (e + (long long)n * 32) * elem;
}

template <typename T>
__global__ void __launch_bounds__(PC_THREADS) potrf_cluster_kernel(Ctx<T> c, const int* __restrict__ pivots,
                                                                   const int* __restrict__ clusters, int count,
                                                                   int smem_bytes, int* fallback) {
    pdl_wait_and_release();
    namespace cgx = cooperative_groups;
    cgx::cluster_group cl = cgx::this_cluster();
    const int CS = (int)cl.num_blocks(), me = (int)cl.block_rank();
    const int item = blockIdx.x / CS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sm = reinterpret_cast<T*>(smem_raw);
    __shared__ int bad;
    __shared__ T Dpc[32 * 33];  // inverse of the current diagonal block, row-major, padded
    // all CTAs of a cluster hold the same pivot, so these exits are uniform over it
    if (item >= count) return;
    const int cid = clusters[item];
    const int n = c.csize[cid];
    const bool fits = pc_need(n, CS, 0, (int)sizeof(T)) <= smem_bytes;
    if (me == 0 && threadIdx.x == 0) fallback[item] = (n > 0 && !fits) ? 1 : 0;
    if (n == 0 || !fits) return;
    T* G = bptr(c, pivots[item]);
    const int gld = c.blk[pivots[item]].ld;
    const int tid = threadIdx.x;
    const int np = (n + 31) / 32;
    // offset of panel p (owned by CTA r = p mod CS) in its owner's shared memory
    auto poff = [&](int p) -> long long {
        long long e = 0;
        for (int q = p % CS; q < p; q += CS) e += (long long)(n - 32 * q) * 32;
        return e;
    };
    long long own = 0;
    for (int p = me; p < np; p += CS) {
        T* P = sm + own;
        const int r0 = 32 * p, ldp = n - r0, w = min(32, n - r0);
        // the panel's rows x w columns (the entries above the diagonal block's diagonal are
        // scratch), eight loads in flight per thread before their stores
        for (int base = 0; base < ldp * w; base += 8 * PC_THREADS) {
            T v[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int idx = base + tid + PC_THREADS * u;
                v[u] = idx < ldp * w ? G[(r0 + idx % ldp) + (size_t)(r0 + idx / ldp) * gld] : T(0);
            }
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int idx = base + tid + PC_THREADS * u;
                if (idx < ldp * w) P[idx] = v[u];  // P[t + j * ldp] with idx = t + j * ldp
            }
        }
        own += (long long)ldp * 32;
    }
    T* S = sm + own;  // staged trailing rows of the current panel
    if (tid == 0) bad = 0;
    __syncthreads();
    bool failed = false;
    for (int p = 0; p < np; p++) {
        const int owner = p % CS;
        const int r0 = 32 * p, ldp = n - r0, w = min(32, n - r0);
        if (owner == me) {
            T* P = sm + poff(p);
            // the diagonal block and its inverse D (into Dpc; D^T also lands in the panel's
            // upper slots, which are not copied back)
            if (tid < 32) chol_diag32(P, ldp, 0, w, Dpc, &bad);
            __syncthreads();
            // rows below: L[t][j] = sum_{l <= j} A[t][l] D[j][l], a warp per four rows, lane = j
            if (!bad) {
                const int lane = tid & 31, wid = tid >> 5;
                for (int t0 = w + 4 * wid; t0 < ldp; t0 += 4 * (PC_THREADS / 32)) {
                    T acc[4] = {T(0), T(0), T(0), T(0)};
                    for (int l = 0; l < w; l++) {
                        const T dl = l <= lane ? Dpc[lane * 33 + l] : T(0);
#pragma unroll
                        for (int u = 0; u < 4; u++)
                            if (t0 + u < ldp) acc[u] += P[(t0 + u) + (size_t)l * ldp] * dl;
                    }
                    __syncwarp();
                    if (lane < w)
#pragma unroll
                        for (int u = 0; u < 4; u++)
                            if (t0 + u < ldp) P[(t0 + u) + (size_t)lane * ldp] = acc[u];
                }
            }
            __syncthreads();
        }
        cl.sync();
        if (*cl.map_shared_rank(&bad, owner)) {
            failed = true;
            break;
        }
        const int rs = r0 + w;  // first trailing row
        if (rs >= n) continue;
        const int ls = n - rs;
        const T* Pp = cl.map_shared_rank(sm, owner) + poff(p);
        // eight distributed-shared-memory loads in flight per thread before their stores (the
        // compiler keeps a load behind an earlier store it cannot tell apart from it)
        for (int base = 0; base < ls * w; base += 8 * PC_THREADS) {
            T v[8];
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const int idx = base + tid + PC_THREADS * j;
                v[j] = T(0);
                if (idx < ls * w) {
                    const int t = idx % ls, k = idx / ls;
                    v[j] = Pp[(rs - r0 + t) + (size_t)k * ldp];
                }
            }
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const int idx = base + tid + PC_THREADS * j;
                if (idx < ls * w) S[idx] = v[j];  // S[t + k * ls] with idx = t + k * ls
            }
        }
        __syncthreads();
        const int rg = tid >> 3, cg = tid & 7;
        for (int q = p + 1 + ((me - (p + 1)) % CS + CS) % CS; q < np; q += CS) {
            T* Q = sm + poff(q);
            const int q0 = 32 * q, ldq = n - q0, wq = min(32, n - q0);
            for (int rb = 0; rb < ldq; rb += 128) {
                T acc[4][4];
#pragma unroll
                for (int u = 0; u < 4; u++)
#pragma unroll
                    for (int v = 0; v < 4; v++) acc[u][v] = T(0);
                for (int k = 0; k < w; k++) {
                    const T* sk = S + (size_t)k * ls;
                    T a[4], b[4];
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const int i = q0 + rb + rg + 32 * u;
                        a[u] = i < n ? sk[i - rs] : T(0);
                    }
#pragma unroll
                    for (int v = 0; v < 4; v++) {
                        const int jj = 4 * cg + v;
                        b[v] = jj < wq ? sk[q0 + jj - rs] : T(0);
                    }
#pragma unroll
                    for (int u = 0; u < 4; u++)
#pragma unroll
                        for (int v = 0; v < 4; v++) acc[u][v] += a[u] * b[v];
                }
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const int t = rb + rg + 32 * u;
#pragma unroll
                    for (int v = 0; v < 4; v++) {
                        const int jj = 4 * cg + v;
                        if (t < ldq && jj < wq && t >= jj) Q[t + (size_t)jj * ldq] -= acc[u][v];
                    }
                }
            }
        }
        __syncthreads();
    }
    // no CTA leaves while another may still read its panels
    cl.sync();
    if (failed) {
        if (me == 0 && tid == 0) atomicCAS(&c.status->not_spd, 0, cid + 1);
        return;
    }
    long long off = 0;
    for (int p = me; p < np; p += CS) {
        const T* P = sm + off;
        const int r0 = 32 * p, ldp = n - r0, w = min(32, n - r0);
        for (int idx = tid; idx < ldp * w; idx += PC_THREADS) {
            const int t = idx % ldp, j = idx / ldp;
            if (t >= j) G[(r0 + t) + (size_t)(r0 + j) * gld] = P[t + (size_t)j * ldp];
        }
        off += (long long)ldp * 32;
    }
}

// ------------------------------------------------------------------------------------
// Inverse of the Cholesky factors, stored transposed in the strictly upper triangle of
// the pivot block: A[j + i*ld] = (L^{-1})[i][j] for i > j (the diagonal, 1/L[i][i], is
// not stored).  One block per 32-column strip of L^{-1}: row blocks of 32 in order, each
// = L_ii^{-1} (E - L[ib, jb:ib] Y[jb:ib]) with the small triangular solves done by warps
// with shuffles.  The strip (n x 32) lives in shared memory.
// ------------------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) trtri_kernel(Ctx<T> c, const int* __restrict__ pivots,
                                                    const int* __restrict__ clusters, const DTile* __restrict__ tiles,
                                                    int ntiles, int smem_elems, long long skip_n2) {
    pdl_wait_and_release();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* Y = reinterpret_cast<T*>(smem_raw);  // Y[i + jj * n], rows i >= jb
    const int t = blockIdx.x;
    if (t >= ntiles || c.status->not_spd) return;
    const int item = tiles[t].item;
    const int cl = clusters[item];
    const int n = c.csize[cl];
    const int jb = tiles[t].tile_i * 32;
    // pivots inverted by potrf3_kernel: those it held in shared memory (potrf_held(n) <=
    // skip_n2) and the large ones
    if (jb >= n || potrf_held(n) <= skip_n2 || (long long)n * 32 > smem_elems) return;
    const int w = min(32, n - jb);
    T* A = bptr(c, pivots[item]);
    const int ld = c.blk[pivots[item]].ld;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5, nty = blockDim.x >> 5;
    // staging of the row block's L tile L[ib:ib+32, jb:ib] (ld 33) where it fits after Y
    T* Lt = Y + (size_t)n * 32;
    const bool stage = (long long)n * 65 <= smem_elems;
    constexpr int TRI_COLS = 4;  // 32 columns over the 8 warps of a 256-thread CTA
    for (int ib = jb; ib < n; ib += 32) {
        const int h = min(32, n - ib);
        const int kw = ib - jb;
        // R = E - L[ib:ib+h, jb:ib] Y[jb:ib, :]: thread (row tx, column group ty) reads each
        // L[i][k] once for its TRI_COLS columns jj = ty + nty u; the tile is first copied to
        // shared memory by the whole CTA (coalesced, many loads in flight)
        if (stage && kw > 0) {
            // eight loads in flight per thread before their stores
            for (int base = 0; base < 32 * kw; base += 8 * 256) {
                T v[8];
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    const int idx = base + threadIdx.x + 256 * u, r = idx & 31, k = idx >> 5;
                    v[u] = (idx < 32 * kw && r < h) ? A[(ib + r) + (size_t)(jb + k) * ld] : T(0);
                }
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    const int idx = base + threadIdx.x + 256 * u;
                    if (idx < 32 * kw) Lt[(idx & 31) + 33 * (idx >> 5)] = v[u];
                }
            }
            __syncthreads();
        }
        if (tx < h) {
            const int i = ib + tx;
            T acc[TRI_COLS];
#pragma unroll
            for (int u = 0; u < TRI_COLS; u++) acc[u] = T(0);
            for (int k = jb; k < ib; k++) {
                const T a0 = stage ? Lt[tx + 33 * (k - jb)] : A[i + (size_t)k * ld];
#pragma unroll
                for (int u = 0; u < TRI_COLS; u++) {
                    const int jj = ty + nty * u;
                    if (jj < w) acc[u] += a0 * Y[k + jj * n];
                }
            }
#pragma unroll
            for (int u = 0; u < TRI_COLS; u++) {
                const int jj = ty + nty * u;
                if (jj < w) Y[i + jj * n] = T(i == jb + jj ? 1 : 0) - acc[u];
            }
        }
        __syncthreads();
        // Y[ib:ib+h, jj] = L_ii^{-1} R[:, jj]: lanes are rows; row ib+tx of the diagonal block
        // in registers; the warp's TRI_COLS columns are substituted together
        T lrow[32];
#pragma unroll
        for (int r = 0; r < 32; r++)
            lrow[r] = (tx < h && r < tx) ? A[(ib + tx) + (size_t)(ib + r) * ld] : T(0);
        const T rdii = tx < h ? T(1) / A[(ib + tx) + (size_t)(ib + tx) * ld] : T(1);
        T acc[TRI_COLS];
#pragma unroll
        for (int u = 0; u < TRI_COLS; u++) {
            const int jj = ty + nty * u;
            acc[u] = (tx < h && jj < w) ? Y[(ib + tx) + jj * n] : T(0);
        }
#pragma unroll
        for (int r = 0; r < 32; r++) {
            if (r < h) {
#pragma unroll
                for (int u = 0; u < TRI_COLS; u++) {
                    const T yr = __shfl_sync(0xffffffffu, acc[u] * rdii, r);
                    if (tx == r) acc[u] = yr;
                    else acc[u] -= lrow[r] * yr;
                }
            }
        }
#pragma unroll
        for (int u = 0; u < TRI_COLS; u++) {
            const int jj = ty + nty * u;
            if (tx < h && jj < w) Y[(ib + tx) + jj * n] = acc[u];
        }
        __syncthreads();
    }
    // strip -> strictly upper triangle, transposed
    for (int jj = ty; jj < w; jj += nty)
        for (int i = jb + jj + 1 + tx; i < n; i += 32) A[(jb + jj) + (size_t)i * ld] = Y[i + jj * n];
}

constexpr int TRB = 32;  // independent indices per TRSM tile

// ------------------------------------------------------------------------------------
// Triangular solves of edge blocks as triangular products with the inverse factor
// (tree.cpp:640-663): out[q][c] = sum_{k<=c} X[q][k] * Linv[c][k], where q runs over the
// independent index (row of B for side 1: B L^{-T}; column of B for side 0: L^{-1} B).
// A tile of 32 independent indices is staged in shared memory; every thread computes
// columns c of one q with four partial sums; no barrier after the staging.
// ------------------------------------------------------------------------------------
// LDLT path (perm_store != nullptr): the s index of B is gathered through the pivot's row
// permutation while the tile is staged: side 0 L^{-1} P^T B, side 1 B P L^{-T}
// (tree.cpp:691-715); such launches always stage (checked when the plan is uploaded).
template <typename T>
__global__ void __launch_bounds__(256) trsm3_kernel(Ctx<T> c, const DTrsm* __restrict__ items,
                                                   const DTile* __restrict__ tiles, int ntiles, int smem_elems,
                                                   const int* __restrict__ perm_store = nullptr,
                                                   const long long* __restrict__ poff = nullptr) {
    pdl_wait_and_release();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* X = reinterpret_cast<T*>(smem_raw);
    const int t = blockIdx.x;
    if (t >= ntiles || c.status->not_spd) return;
    const DTrsm it = items[tiles[t].item];
    const int n = c.csize[it.cluster];
    if (n == 0) return;
    const T* L = bptr(c, it.lblock);
    const int lld = c.blk[it.lblock].ld;
    T* B = bptr(c, it.block);
    const int bld = c.blk[it.block].ld;
    const int m = it.side == 1 ? c.csize[c.blk[it.block].rowc] : c.csize[c.blk[it.block].colc];
    const int r0 = tiles[t].tile_i * TRB;
    if (r0 >= m) return;
    const int tr = min(TRB, m - r0);
    // element (q, k) of B: side 1 B[(r0+q) + k*bld], side 0 B[k + (r0+q)*bld]
    const long long sq = it.side == 1 ? 1 : bld, sk = it.side == 1 ? bld : 1;
    T* Bt = B + (it.side == 1 ? (size_t)r0 : (size_t)r0 * bld);
    // the staged tile is laid out with stride TRB whatever its height tr
    const bool staged = (long long)TRB * n <= smem_elems;
    const int* perm = perm_store ? perm_store + poff[it.cluster] : nullptr;
    const T* src;
    long long xq, xk;
    if (staged) {
        for (int idx = threadIdx.x; idx < tr * n; idx += blockDim.x) {
            int q, k;
            if (it.side == 1) { q = idx % tr; k = idx / tr; } else { k = idx % n; q = idx / n; }
            X[q + k * TRB] = Bt[q * sq + (long long)(perm ? perm[k] : k) * sk];
        }
        __syncthreads();
        src = X;
        xq = 1;
        xk = TRB;
    } else {
        // too large for the shared-memory budget: a copy is needed since B is overwritten
        // column by column; process the columns in decreasing order so that every column
        // is read before it is written (out[., c] needs X[., k <= c] only)
        src = nullptr;
        xq = xk = 0;
    }
    const int q = threadIdx.x % TRB;
    const int sub = threadIdx.x / TRB, lanes = blockDim.x / TRB;
    if (staged) {
        if (q < tr) {
            for (int cc = sub; cc < n; cc += lanes) {
                const T* lrow = L + (size_t)cc * lld;  // (L^{-1})[cc][k] = lrow[k], k < cc
                const T* xr = src + q * xq;
                T s0 = 0, s1 = 0, s2 = 0, s3 = 0;
                int k = 0;
                for (; k + 3 < cc; k += 4) {
                    s0 += xr[k * xk] * lrow[k];
                    s1 += xr[(k + 1) * xk] * lrow[k + 1];
                    s2 += xr[(k + 2) * xk] * lrow[k + 2];
                    s3 += xr[(k + 3) * xk] * lrow[k + 3];
                }
                for (; k < cc; k++) s0 += xr[k * xk] * lrow[k];
                const T diag = xr[cc * xk] / L[cc + (size_t)cc * lld];
                Bt[q * sq + cc * sk] = (s0 + s1) + (s2 + s3) + diag;
            }
        }
    } else {
        // in place from the last column down; one thread group per q, columns in sequence
        if (sub == 0 && q < tr) {
            T* xr = Bt + q * sq;
            for (int cc = n - 1; cc >= 0; cc--) {
                const T* lrow = L + (size_t)cc * lld;
                T s = 0;
                for (int k = 0; k < cc; k++) s += xr[k * sk] * lrow[k];
                xr[cc * sk] = s + xr[cc * sk] / L[cc + (size_t)cc * lld];
            }
        }
    }
}

// The same panel products (LLT pivots, no row permutation) on the tensor cores, FP32 path:
// out = X (L^{-1})^T for a 32-row tile X of the panel, with mma.sync m16n8k8 TF32 tiles and
// FP32 accumulation.  Every operand is split into a TF32 head and a TF32 tail and the
// product summed as head*head + head*tail + tail*head (the "3xTF32" scheme, Ootomo and
// Yokota 2022): about 22 of FP32's 24 significand bits per product (measured 1-4x the SIMT
// kernel's error against FP64).  The tensor core accumulates one 8-deep k-step at a time
// (its internal additions are not rounded to nearest, which over a long inner dimension
// costs accuracy) and the steps are added in FP32 registers.  The tile is staged in shared
// memory with stride TC_XLD (conflict-free A-fragment loads); B fragments come straight
// from the pivot block: B[k][cc] = (L^{-1})[cc][k], the block's column cc above the
// diagonal, 1 / L_cc on it and zero below.  Warp w computes the 8-column blocks w, w + 8,
// ..., each over the k-blocks up to its diagonal.
constexpr int TC_XLD = TRB + 8;

__device__ __forceinline__ uint32_t tf32_of(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ void mma_tf32_16x8x8(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__global__ void __launch_bounds__(256) trsm_tc_kernel(Ctx<float> c, const DTrsm* __restrict__ items,
                                                      const DTile* __restrict__ tiles, int ntiles) {
    pdl_wait_and_release();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* X = reinterpret_cast<float*>(smem_raw);
    const int t = blockIdx.x;
    if (t >= ntiles || c.status->not_spd) return;
    const DTrsm it = items[tiles[t].item];
    const int n = c.csize[it.cluster];
    if (n == 0) return;
    const float* L = bptr(c, it.lblock);
    const int lld = c.blk[it.lblock].ld;
    float* B = bptr(c, it.block);
    const int bld = c.blk[it.block].ld;
    const int m = it.side == 1 ? c.csize[c.blk[it.block].rowc] : c.csize[c.blk[it.block].colc];
    const int r0 = tiles[t].tile_i * TRB;
    if (r0 >= m) return;
    const int tr = min(TRB, m - r0);
    const long long sq = it.side == 1 ? 1 : bld, sk = it.side == 1 ? bld : 1;
    float* Bt = B + (it.side == 1 ? (size_t)r0 : (size_t)r0 * bld);
    const int nc = (n + 7) & ~7;
    for (int idx = threadIdx.x; idx < TRB * nc; idx += blockDim.x) {
        int q, k;
        if (it.side == 1) {
            q = idx % TRB;
            k = idx / TRB;
        } else {
            k = idx % nc;
            q = idx / nc;
        }
        X[q + k * TC_XLD] = (q < tr && k < n) ? Bt[q * sq + (long long)k * sk] : 0.f;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, g = lane >> 2, tg = lane & 3;
    for (int cb = w; cb < nc / 8; cb += 8) {
        const int cc0 = cb * 8, cc = cc0 + g;
        const bool live = cc < n;
        const float* lcol = L + (size_t)(live ? cc : 0) * lld;
        const float dinv = live ? 1.f / lcol[cc] : 0.f;
        float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
        for (int k0 = 0; k0 <= cc0; k0 += 8) {
            const int ka = k0 + tg, kb = ka + 4;
            const float b0 = !live ? 0.f : (ka < cc ? lcol[ka] : (ka == cc ? dinv : 0.f));
            const float b1 = !live ? 0.f : (kb < cc ? lcol[kb] : (kb == cc ? dinv : 0.f));
            uint32_t bh[2] = {tf32_of(b0), tf32_of(b1)};
            uint32_t bl[2] = {tf32_of(b0 - __uint_as_float(bh[0])), tf32_of(b1 - __uint_as_float(bh[1]))};
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const float* xa = X + 16 * h + g;
                const float av[4] = {xa[ka * TC_XLD], xa[8 + ka * TC_XLD], xa[kb * TC_XLD], xa[8 + kb * TC_XLD]};
                uint32_t ah[4], al[4];
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    ah[i] = tf32_of(av[i]);
                    al[i] = tf32_of(av[i] - __uint_as_float(ah[i]));
                }
                // one k-step per tensor-core accumulation (its internal sums are not rounded
                // to nearest); the steps are added in FP32 outside it
                float big[4] = {0.f, 0.f, 0.f, 0.f}, small[4] = {0.f, 0.f, 0.f, 0.f};
                mma_tf32_16x8x8(small, al, bh);
                mma_tf32_16x8x8(small, ah, bl);
                mma_tf32_16x8x8(big, ah, bh);
#pragma unroll
                for (int e = 0; e < 4; e++) acc[h][e] += big[e] + small[e];
            }
        }
#pragma unroll
        for (int h = 0; h < 2; h++)
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int q = 16 * h + g + (i >= 2 ? 8 : 0), col = cc0 + 2 * tg + (i & 1);
                if (q < tr && col < n) Bt[q * sq + (long long)col * sk] = acc[h][i];
            }
    }
}

// The panel products of pivots of at most 32 rows (the thousands of small interface pivots
// of the lowest levels), one warp per 32-row tile, eight tiles per CTA: the same TF32
// head/tail tensor-core products as trsm_tc_kernel, each warp staging its own tile and
// running all of its (at most four) 8-column blocks, so a tile is a warp's work instead of
// a CTA's.
constexpr int TSW = 8;  // tiles (warps) per CTA
__global__ void __launch_bounds__(32 * TSW) trsm_tc_small_kernel(Ctx<float> c, const DTrsm* __restrict__ items,
                                                                  const DTile* __restrict__ tiles, int ntiles) {
    pdl_wait_and_release();
    __shared__ float Xall[TSW][32 * TC_XLD];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int t = blockIdx.x * TSW + wid;
    if (t >= ntiles || c.status->not_spd) return;
    const DTrsm it = items[tiles[t].item];
    const int n = c.csize[it.cluster];
    if (n == 0 || n > 32) return;
    const float* L = bptr(c, it.lblock);
    const int lld = c.blk[it.lblock].ld;
    float* B = bptr(c, it.block);
    const int bld = c.blk[it.block].ld;
    const int m = it.side == 1 ? c.csize[c.blk[it.block].rowc] : c.csize[c.blk[it.block].colc];
    const int r0 = tiles[t].tile_i * TRB;
    if (r0 >= m) return;
    const int tr = min(TRB, m - r0);
    const long long sq = it.side == 1 ? 1 : bld, sk = it.side == 1 ? bld : 1;
    float* Bt = B + (it.side == 1 ? (size_t)r0 : (size_t)r0 * bld);
    const int nc = (n + 7) & ~7;
    float* X = Xall[wid];
    for (int idx = lane; idx < TRB * nc; idx += 32) {
        int q, k;
        if (it.side == 1) {
            q = idx % TRB;
            k = idx / TRB;
        } else {
            k = idx % nc;
            q = idx / nc;
        }
        X[q + k * TC_XLD] = (q < tr && k < n) ? Bt[q * sq + (long long)k * sk] : 0.f;
    }
    __syncwarp();
    const int g = lane >> 2, tg = lane & 3;
    for (int cb = 0; cb < nc / 8; cb++) {
        const int cc0 = cb * 8, cc = cc0 + g;
        const bool live = cc < n;
        const float* lcol = L + (size_t)(live ? cc : 0) * lld;
        const float dinv = live ? 1.f / lcol[cc] : 0.f;
        float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
        for (int k0 = 0; k0 <= cc0; k0 += 8) {
            const int ka = k0 + tg, kb = ka + 4;
            const float b0 = !live ? 0.f : (ka < cc ? lcol[ka] : (ka == cc ? dinv : 0.f));
            const float b1 = !live ? 0.f : (kb < cc ? lcol[kb] : (kb == cc ? dinv : 0.f));
            uint32_t bh[2] = {tf32_of(b0), tf32_of(b1)};
            uint32_t bl[2] = {tf32_of(b0 - __uint_as_float(bh[0])), tf32_of(b1 - __uint_as_float(bh[1]))};
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const float* xa = X + 16 * h + g;
                const float av[4] = {xa[ka * TC_XLD], xa[8 + ka * TC_XLD], xa[kb * TC_XLD], xa[8 + kb * TC_XLD]};
                uint32_t ah[4], al[4];
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    ah[i] = tf32_of(av[i]);
                    al[i] = tf32_of(av[i] - __uint_as_float(ah[i]));
                }
                float big[4] = {0.f, 0.f, 0.f, 0.f}, small[4] = {0.f, 0.f, 0.f, 0.f};
                mma_tf32_16x8x8(small, al, bh);
                mma_tf32_16x8x8(small, ah, bl);
                mma_tf32_16x8x8(big, ah, bh);
#pragma unroll
                for (int e = 0; e < 4; e++) acc[h][e] += big[e] + small[e];
            }
        }
#pragma unroll
        for (int h = 0; h < 2; h++)
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int q = 16 * h + g + (i >= 2 ? 8 : 0), col = cc0 + 2 * tg + (i & 1);
                if (q < tr && col < n) Bt[q * sq + (long long)col * sk] = acc[h][i];
            }
    }
}

// ------------------------------------------------------------------------------------
// General (PLU) path.  Partial-pivot LU of a pivot block (tree.cpp:614-635; getf,
// util.cpp:183-200, in the LAPACK dgetf2 order: the pivot is the first row of largest
// magnitude, the rows are interchanged across the block, the column below is scaled by
// the reciprocal of the pivot, then the rank-1 update), the split of split_LU
// (util.cpp:212-227): L_s = L |D|^1/2, U_s = sign(D) |D|^1/2 D^-1 U, and the inverses of
// both factors for the triangular products of the panels and of the solve:
//   pivot block:   strict lower = L_s, upper with the diagonal = U_s
//   inverse block: strict lower = L_s^{-1}, upper with the diagonal = U_s^{-1}
//                  (diag L_s^{-1} = |diag U_s^{-1}|, not stored)
//   perm[i]: the row of the pivot block that is row i of P^T A (swap2perm, util.cpp:76-88);
//   swp[j]: the row interchanged with row j at step j (both at the cluster's offset poff)
// One CTA per pivot.  The block is worked on in shared memory when n^2 + n elements fit,
// else in the inverse block in global memory (n elements of shared memory).
// ------------------------------------------------------------------------------------
constexpr int LU_THREADS = 256;

template <typename T>
__device__ __forceinline__ void argmax_merge(T& v, int& i, T ov, int oi) {
    if (ov > v || (ov == v && oi < i)) {
        v = ov;
        i = oi;
    }
}

template <typename T>
__global__ void __launch_bounds__(LU_THREADS) getrf_kernel(Ctx<T> c, const int* __restrict__ pivots,
                                                          const int* __restrict__ invs,
                                                          const int* __restrict__ clusters, int count, int smem_elems,
                                                          int* __restrict__ perm_store, int* __restrict__ swp_store,
                                                          const long long* __restrict__ poff) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ T wv[LU_THREADS / 32];
    __shared__ int wi[LU_THREADS / 32];
    __shared__ int prow, bad;
    const int item = blockIdx.x;
    if (item >= count || c.status->not_spd) return;
    const int cid = clusters[item];
    const int n = c.csize[cid];
    if (n == 0) return;
    T* G = bptr(c, pivots[item]);
    const int gld = c.blk[pivots[item]].ld;
    T* Wg = bptr(c, invs[item]);
    const int wld = c.blk[invs[item]].ld;
    T* tmp = reinterpret_cast<T*>(smem_raw);
    const bool in_smem = (long long)n * n + n <= smem_elems;
    T* A = in_smem ? tmp + n : Wg;
    const int lda = in_smem ? n : wld;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    int* swp = swp_store + poff[cid];
    int* perm = perm_store + poff[cid];
    for (int idx = tid; idx < n * n; idx += LU_THREADS) {
        const int i = idx % n, j = idx / n;
        A[i + (size_t)j * lda] = G[i + (size_t)j * gld];
    }
    if (tid == 0) bad = 0;
    __syncthreads();
    for (int j = 0; j < n; j++) {
        T bv = T(-1);
        int bi = n;
        for (int i = j + tid; i < n; i += LU_THREADS) argmax_merge(bv, bi, (T)fabs(A[i + (size_t)j * lda]), i);
        for (int o = 16; o > 0; o >>= 1) {
            const T ov = __shfl_down_sync(0xffffffffu, bv, o);
            const int oi = __shfl_down_sync(0xffffffffu, bi, o);
            argmax_merge(bv, bi, ov, oi);
        }
        if (lane == 0) {
            wv[wid] = bv;
            wi[wid] = bi;
        }
        __syncthreads();
        if (tid == 0) {
            T v = wv[0];
            int i = wi[0];
            for (int w = 1; w < LU_THREADS / 32; w++) argmax_merge(v, i, wv[w], wi[w]);
            prow = i;
            swp[j] = i;
            if (A[i + (size_t)j * lda] == T(0)) bad = 1;  // singular pivot (getf info > 0)
        }
        __syncthreads();
        if (bad) break;
        const int p = prow;
        if (p != j)
            for (int col = tid; col < n; col += LU_THREADS) {
                const T a = A[j + (size_t)col * lda];
                A[j + (size_t)col * lda] = A[p + (size_t)col * lda];
                A[p + (size_t)col * lda] = a;
            }
        __syncthreads();
        const T d = T(1) / A[j + (size_t)j * lda];
        for (int i = j + 1 + tid; i < n; i += LU_THREADS) A[i + (size_t)j * lda] *= d;
        __syncthreads();
        const int m = n - j - 1;
        for (int idx = tid; idx < m * m; idx += LU_THREADS) {
            const int i = j + 1 + idx % m, col = j + 1 + idx / m;
            A[i + (size_t)col * lda] -= A[i + (size_t)j * lda] * A[j + (size_t)col * lda];
        }
        __syncthreads();
    }
    if (bad) {
        if (tid == 0) atomicCAS(&c.status->not_spd, 0, cid + 1);
        return;
    }
    if (tid == 0) {
        for (int i = 0; i < n; i++) perm[i] = i;
        for (int i = 0; i < n; i++) {
            const int s = swp[i], t = perm[s];
            perm[s] = perm[i];
            perm[i] = t;
        }
    }
    // split_LU: off-diagonal entries from the unsplit diagonal, then the diagonal
    for (int idx = tid; idx < n * n; idx += LU_THREADS) {
        const int i = idx % n, j = idx / n;
        if (i == j) continue;
        T& a = A[i + (size_t)j * lda];
        if (i > j) {
            a = a * dsqrt((T)fabs(A[j + (size_t)j * lda]));
        } else {
            const T di = A[i + (size_t)i * lda];
            const T sg = T((di > T(0)) - (di < T(0)));
            a = sg * dsqrt((T)fabs(di)) * (a / di);
        }
    }
    __syncthreads();
    for (int j = tid; j < n; j += LU_THREADS) {
        T& d = A[j + (size_t)j * lda];
        const T sg = T((d > T(0)) - (d < T(0)));
        d = sg * dsqrt((T)fabs(d));
    }
    __syncthreads();
    for (int idx = tid; idx < n * n; idx += LU_THREADS) {
        const int i = idx % n, j = idx / n;
        G[i + (size_t)j * gld] = A[i + (size_t)j * lda];
    }
    __syncthreads();
    // L_s^{-1} in the strict lower triangle, columns from the last: with L_s = [l x; 0 L22]
    // partitioned at j, column j of the inverse below the diagonal is -L22^{-1} x / l
    // (L_s(i,i) = |U_s(i,i)|, still on the diagonal)
    for (int j = n - 1; j >= 0; j--) {
        const int m = n - j - 1;
        for (int i = tid; i < m; i += LU_THREADS) tmp[i] = A[(j + 1 + i) + (size_t)j * lda];
        __syncthreads();
        const T lj = T(1) / (T)fabs(A[j + (size_t)j * lda]);
        for (int i = j + 1 + tid; i < n; i += LU_THREADS) {
            T s = tmp[i - j - 1] / (T)fabs(A[i + (size_t)i * lda]);
            for (int k = j + 1; k < i; k++) s += A[i + (size_t)k * lda] * tmp[k - j - 1];
            A[i + (size_t)j * lda] = -lj * s;
        }
        __syncthreads();
    }
    // U_s^{-1} in the upper triangle, columns from the first (LAPACK dtrti2 order)
    for (int j = 0; j < n; j++) {
        for (int i = tid; i < j; i += LU_THREADS) tmp[i] = A[i + (size_t)j * lda];
        if (tid == 0) A[j + (size_t)j * lda] = T(1) / A[j + (size_t)j * lda];
        __syncthreads();
        const T uj = A[j + (size_t)j * lda];
        for (int i = tid; i < j; i += LU_THREADS) {
            T s = 0;
            for (int k = i; k < j; k++) s += A[i + (size_t)k * lda] * tmp[k];
            A[i + (size_t)j * lda] = -uj * s;
        }
        __syncthreads();
    }
    if (in_smem)
        for (int idx = tid; idx < n * n; idx += LU_THREADS) {
            const int i = idx % n, j = idx / n;
            Wg[i + (size_t)j * wld] = A[i + (size_t)j * lda];
        }
}

// Panels of the PLU path (tree.cpp:668-689): in-edge blocks B <- L_s^{-1} P^T B (side 0),
// out-edge blocks B <- B U_s^{-1} (side 1), as triangular products with the inverse block
// (DTrsm::lblock).  Tiles of 32 independent indices as in trsm3_kernel; the rows of a
// side-0 tile are gathered through perm while it is staged.  Blocks too large for the
// shared-memory budget: one thread per index, in place (rows interchanged first).
template <typename T>
__global__ void __launch_bounds__(256) lu_trsm_kernel(Ctx<T> c, const DTrsm* __restrict__ items,
                                                     const DTile* __restrict__ tiles, int ntiles, int smem_elems,
                                                     const int* __restrict__ perm_store,
                                                     const int* __restrict__ swp_store,
                                                     const long long* __restrict__ poff) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* X = reinterpret_cast<T*>(smem_raw);
    const int t = blockIdx.x;
    if (t >= ntiles || c.status->not_spd) return;
    const DTrsm it = items[tiles[t].item];
    const int n = c.csize[it.cluster];
    if (n == 0) return;
    const T* W = bptr(c, it.lblock);
    const int wld = c.blk[it.lblock].ld;
    T* B = bptr(c, it.block);
    const int bld = c.blk[it.block].ld;
    const int m = it.side == 1 ? c.csize[c.blk[it.block].rowc] : c.csize[c.blk[it.block].colc];
    const int r0 = tiles[t].tile_i * TRB;
    if (r0 >= m) return;
    const int tr = min(TRB, m - r0);
    const long long sq = it.side == 1 ? 1 : bld, sk = it.side == 1 ? bld : 1;
    T* Bt = B + (it.side == 1 ? (size_t)r0 : (size_t)r0 * bld);
    const int* perm = perm_store + poff[it.cluster];
    const int q = threadIdx.x % TRB, sub = threadIdx.x / TRB, lanes = blockDim.x / TRB;
    if ((long long)TRB * n <= smem_elems) {  // the tile's stride is TRB whatever its height tr
        for (int idx = threadIdx.x; idx < tr * n; idx += blockDim.x) {
            int qq, k;
            if (it.side == 1) {
                qq = idx % tr;
                k = idx / tr;
            } else {
                k = idx % n;
                qq = idx / n;
            }
            const int kr = it.side == 1 ? k : perm[k];
            X[qq + k * TRB] = Bt[qq * sq + (long long)kr * sk];
        }
        __syncthreads();
        if (q < tr) {
            const T* xr = X + q;
            for (int cc = sub; cc < n; cc += lanes) {
                T s0 = 0, s1 = 0;
                if (it.side == 0) {
                    int k = 0;
                    for (; k + 1 < cc; k += 2) {
                        s0 += W[cc + (size_t)k * wld] * xr[k * TRB];
                        s1 += W[cc + (size_t)(k + 1) * wld] * xr[(k + 1) * TRB];
                    }
                    for (; k < cc; k++) s0 += W[cc + (size_t)k * wld] * xr[k * TRB];
                    s0 += (T)fabs(W[cc + (size_t)cc * wld]) * xr[cc * TRB];
                } else {
                    const T* wc = W + (size_t)cc * wld;
                    int k = 0;
                    for (; k + 1 <= cc; k += 2) {
                        s0 += xr[k * TRB] * wc[k];
                        s1 += xr[(k + 1) * TRB] * wc[k + 1];
                    }
                    for (; k <= cc; k++) s0 += xr[k * TRB] * wc[k];
                }
                Bt[q * sq + (long long)cc * sk] = s0 + s1;
            }
        }
    } else if (sub == 0 && q < tr) {
        T* xr = Bt + q * sq;
        if (it.side == 0) {
            const int* swp = swp_store + poff[it.cluster];
            for (int i = 0; i < n; i++) {
                const int s = swp[i];
                if (s != i) {
                    const T a = xr[i * sk];
                    xr[i * sk] = xr[s * sk];
                    xr[s * sk] = a;
                }
            }
            for (int cc = n - 1; cc >= 0; cc--) {
                T s = (T)fabs(W[cc + (size_t)cc * wld]) * xr[cc * sk];
                for (int k = 0; k < cc; k++) s += W[cc + (size_t)k * wld] * xr[k * sk];
                xr[cc * sk] = s;
            }
        } else {
            for (int cc = n - 1; cc >= 0; cc--) {
                const T* wc = W + (size_t)cc * wld;
                T s = 0;
                for (int k = 0; k <= cc; k++) s += xr[k * sk] * wc[k];
                xr[cc * sk] = s;
            }
        }
    }
}

// ------------------------------------------------------------------------------------
// LDLT path.  Eigen's pivoted LDL^T of a pivot block (util.cpp:167-184 over
// Eigen/src/Cholesky/LDLT.h, ldlt_inplace<Lower>::unblocked): at step k the pivot is the
// first diagonal entry of largest magnitude among k..n-1 as they stand (those after k not
// yet updated), swapped symmetrically inside the lower triangle, then the left-looking
// column update.  L_s = L |D|^1/2, s = sign(D), perm = swap2perm(transpositions); the
// block is left in the Cholesky path's layout (L_s in the lower triangle, (L_s^{-1})^T in
// the strict upper triangle), so the TRSM and solve kernels of that path apply.  newpiv
// (scaling): receives diag(s), the cluster's new pivot (tree.cpp:830).  One CTA per pivot;
// shared memory when n^2 + n elements fit, else in place in the pivot block.
// ------------------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(LU_THREADS) ldlt_kernel(Ctx<T> c, const int* __restrict__ pivots,
                                                         const int* __restrict__ clusters,
                                                         const int* __restrict__ newpiv, int count, int smem_elems,
                                                         int* __restrict__ perm_store, int* __restrict__ swp_store,
                                                         T* __restrict__ sign_store,
                                                         const long long* __restrict__ poff) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ T wv[LU_THREADS / 32];
    __shared__ int wi[LU_THREADS / 32];
    __shared__ T red[33];
    __shared__ T s_gmax;
    __shared__ int prow, bad, zero_seen;
    const int item = blockIdx.x;
    if (item >= count || c.status->not_spd) return;
    const int cid = clusters[item];
    const int n = c.csize[cid];
    if (n == 0) return;
    T* G = bptr(c, pivots[item]);
    const int gld = c.blk[pivots[item]].ld;
    T* tmp = reinterpret_cast<T*>(smem_raw);
    const bool in_smem = (long long)n * n + n <= smem_elems;
    T* A = in_smem ? tmp + n : G;
    const int lda = in_smem ? n : gld;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    int* swp = swp_store + poff[cid];
    int* perm = perm_store + poff[cid];
    T* sg = sign_store + poff[cid];
    if (in_smem)
        for (int idx = tid; idx < n * n; idx += LU_THREADS) {
            const int i = idx % n, j = idx / n;
            if (i >= j) A[i + (size_t)j * lda] = G[i + (size_t)j * gld];
        }
    if (tid == 0) {
        bad = 0;
        zero_seen = 0;
    }
    __syncthreads();
    for (int k = 0; k < n; k++) {
        // pivot: the first diagonal entry of largest magnitude among k..n-1
        T bv = T(-1);
        int bi = n;
        for (int j = k + tid; j < n; j += LU_THREADS) argmax_merge(bv, bi, (T)fabs(A[j + (size_t)j * lda]), j);
        for (int o = 16; o > 0; o >>= 1) {
            const T ov = __shfl_down_sync(0xffffffffu, bv, o);
            const int oi = __shfl_down_sync(0xffffffffu, bi, o);
            argmax_merge(bv, bi, ov, oi);
        }
        if (lane == 0) {
            wv[wid] = bv;
            wi[wid] = bi;
        }
        __syncthreads();
        if (tid == 0) {
            T v = wv[0];
            int i = wi[0];
            for (int w = 1; w < LU_THREADS / 32; w++) argmax_merge(v, i, wv[w], wi[w]);
            s_gmax = v;
        }
        __syncthreads();
        {
            // the first entry within the tie window of the largest (the oracle's rule)
            const T thr = s_gmax * (T(1) - qrcp_tie<T>());
            int f = n;
            for (int j = k + tid; j < n; j += LU_THREADS)
                if ((T)fabs(A[j + (size_t)j * lda]) >= thr) {
                    f = j;
                    break;
                }
            for (int o = 16; o > 0; o >>= 1) f = min(f, __shfl_down_sync(0xffffffffu, f, o));
            if (lane == 0) wi[wid] = f;
            __syncthreads();
            if (tid == 0) {
                int i = wi[0];
                for (int w = 1; w < LU_THREADS / 32; w++) i = min(i, wi[w]);
                if (i >= n) i = k;
                prow = i;
                swp[k] = i;
            }
            __syncthreads();
        }
        const int big = prow;
        if (big != k) {
            // symmetric swap inside the lower triangle: row k / row big left of column k,
            // columns k / big below row big, the two diagonals, and the entries between
            for (int q = tid; q < n; q += LU_THREADS) {
                if (q < k) {
                    const T a = A[k + (size_t)q * lda];
                    A[k + (size_t)q * lda] = A[big + (size_t)q * lda];
                    A[big + (size_t)q * lda] = a;
                } else if (q > big) {
                    const T a = A[q + (size_t)k * lda];
                    A[q + (size_t)k * lda] = A[q + (size_t)big * lda];
                    A[q + (size_t)big * lda] = a;
                } else if (q == k) {
                    const T a = A[k + (size_t)k * lda];
                    A[k + (size_t)k * lda] = A[big + (size_t)big * lda];
                    A[big + (size_t)big * lda] = a;
                } else if (q < big) {  // k < q < big
                    const T a = A[q + (size_t)k * lda];
                    A[q + (size_t)k * lda] = A[big + (size_t)q * lda];
                    A[big + (size_t)q * lda] = a;
                }
            }
            __syncthreads();
        }
        // left-looking update of column k: temp_j = D_j A(k,j), A(k,k) -= A(k,:) temp,
        // A(k+1:,k) -= A(k+1:,0:k) temp
        if (k > 0) {
            for (int j = tid; j < k; j += LU_THREADS) tmp[j] = A[j + (size_t)j * lda] * A[k + (size_t)j * lda];
            __syncthreads();
            T part = 0;
            for (int j = tid; j < k; j += LU_THREADS) part += A[k + (size_t)j * lda] * tmp[j];
            part = block_sum(part, red);
            for (int i = k + 1 + tid; i < n; i += LU_THREADS) {
                T s = 0;
                for (int j = 0; j < k; j++) s += A[i + (size_t)j * lda] * tmp[j];
                A[i + (size_t)k * lda] -= s;
            }
            if (tid == 0) A[k + (size_t)k * lda] -= part;
            __syncthreads();
        }
        const T akk = A[k + (size_t)k * lda];
        const bool valid = fabs(akk) > T(0);
        if (k == 0 && !valid) {
            if (tid == 0) bad = 1;
            break;
        }
        int nz = 0;
        for (int i = k + 1 + tid; i < n; i += LU_THREADS) {
            if (valid) A[i + (size_t)k * lda] /= akk;
            else nz |= A[i + (size_t)k * lda] != T(0);
        }
        if (nz) bad = 1;
        __syncthreads();
        if (tid == 0) {
            if (zero_seen && valid) bad = 1;
            else if (!valid) zero_seen = 1;
        }
        __syncthreads();
    }
    __syncthreads();
    if (bad) {
        if (tid == 0) atomicCAS(&c.status->not_spd, 0, cid + 1);
        return;
    }
    if (tid == 0) {
        for (int i = 0; i < n; i++) perm[i] = i;
        for (int i = 0; i < n; i++) {
            const int s = swp[i], t = perm[s];
            perm[s] = perm[i];
            perm[i] = t;
        }
    }
    // L_s = L |D|^1/2 below the diagonal from the unscaled diagonal, then the diagonal
    for (int idx = tid; idx < n * n; idx += LU_THREADS) {
        const int i = idx % n, j = idx / n;
        if (i > j) A[i + (size_t)j * lda] *= dsqrt((T)fabs(A[j + (size_t)j * lda]));
    }
    __syncthreads();
    for (int j = tid; j < n; j += LU_THREADS) {
        T& d = A[j + (size_t)j * lda];
        sg[j] = T((d > T(0)) - (d < T(0)));
        d = dsqrt((T)fabs(d));
    }
    __syncthreads();
    // (L_s^{-1})^T into the strict upper triangle, columns of L_s^{-1} from the last:
    // column j below the diagonal = -L22^{-1} x / l_jj, L22^{-1} read back from the
    // upper triangle (diagonal 1 / L_s(i,i))
    for (int j = n - 1; j >= 0; j--) {
        const T lj = T(1) / A[j + (size_t)j * lda];
        for (int i = j + 1 + tid; i < n; i += LU_THREADS) {
            T s = A[i + (size_t)j * lda] / A[i + (size_t)i * lda];
            for (int k = j + 1; k < i; k++) s += A[k + (size_t)i * lda] * A[k + (size_t)j * lda];
            A[j + (size_t)i * lda] = -lj * s;
        }
        __syncthreads();
    }
    if (in_smem)
        for (int idx = tid; idx < n * n; idx += LU_THREADS) {
            const int i = idx % n, j = idx / n;
            G[i + (size_t)j * gld] = A[i + (size_t)j * lda];
        }
    if (newpiv) {
        T* Np = bptr(c, newpiv[item]);
        const int nld = c.blk[newpiv[item]].ld;
        for (int j = tid; j < n; j += LU_THREADS) Np[j + (size_t)j * nld] = sg[j];
    }
}

// LDLT sparsification with a sign pivot (tree.cpp:1069-1097): the pivot block of the
// cluster (diag(s) from its scaling) becomes M = Q^T D Q (the rows first, piv Q, then the
// columns, Q^T piv, as the reference's two ormqr calls), then splits: M[0:k, 0:k] stays
// as the cluster's pivot, M[k:r, k:r] becomes the sibling's pivot, M[k:r, 0:k] the block
// of the edge cluster -> sibling; the sibling's size is r - k.  Reflector j: 1 at row j,
// V[j+1:r, j] below, tau from the QRCP.  One CTA per sparsified cluster.
template <typename T>
__global__ void __launch_bounds__(256) pivot_split_kernel(Ctx<T> c, const DSpars* __restrict__ items,
                                                          const int* __restrict__ sib_of,
                                                          const int* __restrict__ sib_piv_of,
                                                          const int* __restrict__ aso_of,
                                                          const int* __restrict__ piv_of, const T* vstore,
                                                          const T* taus, const T* __restrict__ sign_store,
                                                          const long long* __restrict__ soff) {
    const DSpars it = items[blockIdx.x];
    if (c.status->not_spd) return;
    const int cl = it.cluster;
    const int r = c.rows0[cl], k = c.csize[cl];
    const int sib = sib_of[blockIdx.x];
    if (k >= r) {
        if (threadIdx.x == 0) c.csize[sib] = c.rows0[sib] = 0;
        return;
    }
    T* M = bptr(c, piv_of[blockIdx.x]);
    const int ld = c.blk[piv_of[blockIdx.x]].ld;
    const int vld = c.cap[cl];
    const T* V = vstore + it.v_off;
    const T* tau = taus + it.tau_off;
    // the oracle's deviation: signs all equal -> Q^T D Q = D exactly, kept as it is
    const T* sg = sign_store + soff[cl];
    int uni = 1;
    for (int p = threadIdx.x; p < r; p += blockDim.x) uni &= sg[p] == sg[0];
    const bool all_uniform = __syncthreads_and(uni);
    // rows: M[p, :] <- M[p, :] H_0 H_1 ... H_{k-1}
    for (int p = threadIdx.x; p < r && !all_uniform; p += blockDim.x)
        for (int j = 0; j < k; j++) {
            const T tj = tau[j];
            if (tj == T(0)) continue;
            T w = M[p + (size_t)j * ld];
            for (int q = j + 1; q < r; q++) w += M[p + (size_t)q * ld] * V[q + (size_t)j * vld];
            w *= tj;
            M[p + (size_t)j * ld] -= w;
            for (int q = j + 1; q < r; q++) M[p + (size_t)q * ld] -= w * V[q + (size_t)j * vld];
        }
    __syncthreads();
    // columns: M[:, q] <- H_{k-1} ... H_0 M[:, q]
    for (int q = threadIdx.x; q < r && !all_uniform; q += blockDim.x) {
        T* m = M + (size_t)q * ld;
        for (int j = 0; j < k; j++) {
            const T tj = tau[j];
            if (tj == T(0)) continue;
            T w = m[j];
            for (int i = j + 1; i < r; i++) w += V[i + (size_t)j * vld] * m[i];
            w *= tj;
            m[j] -= w;
            for (int i = j + 1; i < r; i++) m[i] -= w * V[i + (size_t)j * vld];
        }
    }
    __syncthreads();
    T* S = bptr(c, sib_piv_of[blockIdx.x]);
    const int sld = c.blk[sib_piv_of[blockIdx.x]].ld;
    T* E = bptr(c, aso_of[blockIdx.x]);
    const int eld = c.blk[aso_of[blockIdx.x]].ld;
    const int m = r - k;
    for (int idx = threadIdx.x; idx < m * r; idx += blockDim.x) {
        const int i = idx % m, j = idx / m;  // row k + i, column j
        const T v = M[(k + i) + (size_t)j * ld];
        if (j < k) E[i + (size_t)j * eld] = v;
        else S[i + (size_t)(j - k) * sld] = v;
    }
    if (threadIdx.x == 0) c.csize[sib] = c.rows0[sib] = m;
}

// ------------------------------------------------------------------------------------
// Schur complement updates grouped by target block, applied in the reference order
// (tree.cpp:748-793, 858-883): C(n1 x n2) -= op1(B1) op2(B2).  32x32 output tile per
// block, 256 threads, 2x2 outputs per thread, K staged through shared memory.
// ------------------------------------------------------------------------------------
constexpr int ST = 32;
constexpr int SK = 16;

// LDLT path (signs != nullptr): C -= op(B1) D^{-1} op(B2) with D = diag(sign) of the
// eliminated cluster s (tree.cpp:784-789; the signs are +-1, so D^{-1} = D).
template <typename T>
__global__ void __launch_bounds__(256) schur_kernel(Ctx<T> c, const DTarget* __restrict__ targets,
                                                     const DUpd* __restrict__ ups, const DTile* __restrict__ tiles,
                                                     int ntiles, const T* __restrict__ signs = nullptr,
                                                     const long long* __restrict__ soff = nullptr) {
    pdl_wait_and_release();
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
                if (i < M && k < S) {
                    v = up.t1 ? B1[k + (size_t)i * ld1] : B1[i + (size_t)k * ld1];
                    if (signs) v *= signs[soff[up.s] + k];
                }
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

// The Schur updates on the tensor cores, FP32 path: the same 32x32 tiles of C, X and Y
// staged SKT = 32 entries of the inner dimension at a time (LDLT signs applied);
// warp w owns the 16x8 piece (rows 16 (w mod 2), columns 8 (w / 2)) and accumulates
// -X Y into it with mma.sync m16n8k8 TF32, each operand split into TF32 head and tail
// (head*head + head*tail + tail*head, close to FP32 accuracy), four k-steps per staged
// chunk.
constexpr int SKT = 32;
__global__ void __launch_bounds__(256) schur_tc_kernel(Ctx<float> c, const DTarget* __restrict__ targets,
                                                       const DUpd* __restrict__ ups, const DTile* __restrict__ tiles,
                                                       int ntiles, const float* __restrict__ signs = nullptr,
                                                       const long long* __restrict__ soff = nullptr) {
    pdl_wait_and_release();
    const int t = blockIdx.x;
    if (t >= ntiles || c.status->not_spd) return;
    const DTarget tg = targets[tiles[t].item];
    const DBlock cb = c.blk[tg.target];
    const int M = c.csize[cb.rowc], N = c.csize[cb.colc];
    const int i0 = tiles[t].tile_i * ST, j0 = tiles[t].tile_j * ST;
    if (i0 >= M || j0 >= N) return;
    if (tg.syrk && i0 + ST <= j0) return;  // strictly upper tile
    __shared__ float Xs[ST][SKT + 4];
    __shared__ float Ys[SKT][ST + 8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, g = lane >> 2, tq = lane & 3;
    const int mh = 16 * (w & 1), nb = 8 * (w >> 1);
    float* C = c.arena + cb.off;
    const int ldc = cb.ld;
    float acc[4];
#pragma unroll
    for (int e = 0; e < 4; e++) {
        const int i = i0 + mh + g + (e >= 2 ? 8 : 0), j = j0 + nb + 2 * tq + (e & 1);
        acc[e] = (i < M && j < N) ? C[i + (size_t)j * ldc] : 0.f;
    }
    for (int u = 0; u < tg.count; u++) {
        const DUpd up = ups[tg.first + u];
        const int S = c.csize[up.s];
        const float* B1 = bptr(c, up.b1);
        const int ld1 = c.blk[up.b1].ld;
        const float* B2 = bptr(c, up.b2);
        const int ld2 = c.blk[up.b2].ld;
        for (int k0 = 0; k0 < S; k0 += SKT) {
            for (int idx = threadIdx.x; idx < ST * SKT; idx += 256) {
                int ii, kk;
                if (up.t1) { kk = idx % SKT; ii = idx / SKT; } else { ii = idx % ST; kk = idx / ST; }
                const int i = i0 + ii, k = k0 + kk;
                float v = 0.f;
                if (i < M && k < S) {
                    v = up.t1 ? B1[k + (size_t)i * ld1] : B1[i + (size_t)k * ld1];
                    if (signs) v *= signs[soff[up.s] + k];
                }
                Xs[ii][kk] = v;
            }
            for (int idx = threadIdx.x; idx < ST * SKT; idx += 256) {
                int jj, kk;
                if (up.t2) { jj = idx % ST; kk = idx / ST; } else { kk = idx % SKT; jj = idx / SKT; }
                const int j = j0 + jj, k = k0 + kk;
                float v = 0.f;
                if (j < N && k < S) v = up.t2 ? B2[j + (size_t)k * ld2] : B2[k + (size_t)j * ld2];
                Ys[kk][jj] = v;
            }
            __syncthreads();
#pragma unroll
            for (int ks = 0; ks < SKT; ks += 8) {
                // A = -X (rows mh.., inner ks..), B = Y (inner ks.., columns nb..)
                const float av[4] = {-Xs[mh + g][ks + tq], -Xs[mh + g + 8][ks + tq], -Xs[mh + g][ks + tq + 4],
                                     -Xs[mh + g + 8][ks + tq + 4]};
                const float bv[2] = {Ys[ks + tq][nb + g], Ys[ks + tq + 4][nb + g]};
                uint32_t ah[4], al[4], bh[2], bl[2];
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    ah[e] = tf32_of(av[e]);
                    al[e] = tf32_of(av[e] - __uint_as_float(ah[e]));
                }
#pragma unroll
                for (int e = 0; e < 2; e++) {
                    bh[e] = tf32_of(bv[e]);
                    bl[e] = tf32_of(bv[e] - __uint_as_float(bh[e]));
                }
                // one k-step per tensor-core accumulation, the steps added in FP32 outside it
                float big[4] = {0.f, 0.f, 0.f, 0.f}, small[4] = {0.f, 0.f, 0.f, 0.f};
                mma_tf32_16x8x8(small, al, bh);
                mma_tf32_16x8x8(small, ah, bl);
                mma_tf32_16x8x8(big, ah, bh);
#pragma unroll
                for (int e = 0; e < 4; e++) acc[e] += big[e] + small[e];
            }
            __syncthreads();
        }
    }
#pragma unroll
    for (int e = 0; e < 4; e++) {
        const int i = i0 + mh + g + (e >= 2 ? 8 : 0), j = j0 + nb + 2 * tq + (e & 1);
        if (i < M && j < N && (!tg.syrk || i >= j)) C[i + (size_t)j * ldc] = acc[e];
    }
}

// ------------------------------------------------------------------------------------
// Sparsification (tree.cpp:1189-1224, 1292-1347, 980-1104)
// ------------------------------------------------------------------------------------
// The sparsification QRCP (Asn = [A_sn (in-edges) | A_ns^T (out-edges)], rows = size(c))
// lives in qrcp.cu; its output (R, reflectors, pivot vector and inverse, tau, rank) lands
// in the workspace ws at the matrix's offset, ld = cap(c), columns in position order.


// Blocked compact WY form of Q = H_0 ... H_{k-1}: reflectors in blocks of QB = 32,
// Q = Q_0 Q_1 ..., Q_b = I - V_b T_b V_b^T with T_b the 32x32 upper triangular factor of
// block b (LAPACK dlarft, forward, columnwise, per block):
//   T_b[i][i] = tau_i,  T_b[j][i] = -tau_i sum_{l=j}^{i-1} T_b[j][l] Z_b[l][i]  (j < i),
// Z_b = V_b^T V_b (V_b unit lower trapezoidal).  Phase 1: one pass over the rows of up to
// LB_GROUP blocks, staged LB_ROWS rows at a time in shared memory; thread (w, lane) sums
// Z_b[w + 8q][lane], q < 4, for every block of the group.  Phase 2: warp b runs the
// 32-step recurrence of block b with row j of T_b in lane j's registers and column i of
// Z_b in lane i's registers.  T_b goes to the diagonal block b of the k x k T store (ld
// ldt).  256 threads; sm holds larft_smem_elems() elements.
constexpr int QB = 32;
constexpr int LB_GROUP = 8;
constexpr int LB_ROWS = 32;
constexpr int LB_LD = LB_GROUP * QB + 1;
__host__ __device__ constexpr int larft_smem_elems() {
    return LB_ROWS * LB_LD > LB_GROUP * QB * (QB + 1) ? LB_ROWS * LB_LD : LB_GROUP * QB * (QB + 1);
}

template <typename T>
__device__ void larft_blocks(const T* V, int ldv, int rows, int k, const T* tau, T* Tm, int ldt, T* sm) {
    const int tid = threadIdx.x, nth = blockDim.x;
    const int lane = tid & 31, w = tid >> 5;
    const int nb = (k + QB - 1) / QB;
    for (int g0 = 0; g0 < nb; g0 += LB_GROUP) {
        const int gb = min(LB_GROUP, nb - g0);
        const int c0 = g0 * QB, gw = gb * QB;
        T acc[LB_GROUP][4];
#pragma unroll
        for (int b = 0; b < LB_GROUP; b++)
#pragma unroll
            for (int q = 0; q < 4; q++) acc[b][q] = T(0);
        for (int r0 = c0; r0 < rows; r0 += LB_ROWS) {
            __syncthreads();
            for (int idx = tid; idx < LB_ROWS * gw; idx += nth) {
                const int rr = idx % LB_ROWS, cc = idx / LB_ROWS;
                const int r = r0 + rr, j = c0 + cc;
                T v = T(0);
                if (r < rows && j < k) v = r > j ? V[r + (size_t)j * ldv] : (r == j ? T(1) : T(0));
                sm[rr * LB_LD + cc] = v;
            }
            __syncthreads();
            const int nr = min(LB_ROWS, rows - r0);
            for (int rr = 0; rr < nr; rr++) {
                const T* tr = sm + rr * LB_LD;
#pragma unroll
                for (int b = 0; b < LB_GROUP; b++) {
                    if (b < gb) {
                        const T vi = tr[b * QB + lane];
#pragma unroll
                        for (int q = 0; q < 4; q++) acc[b][q] += tr[b * QB + w + 8 * q] * vi;
                    }
                }
            }
        }
        __syncthreads();
#pragma unroll
        for (int b = 0; b < LB_GROUP; b++)
            if (b < gb)
#pragma unroll
                for (int q = 0; q < 4; q++) sm[(b * QB + w + 8 * q) * (QB + 1) + lane] = acc[b][q];
        __syncthreads();
        if (w < gb) {
            const int i0 = c0 + w * QB, bw = min(QB, k - i0);
            T zc[QB], trow[QB];
#pragma unroll
            for (int l = 0; l < QB; l++) {
                zc[l] = sm[(w * QB + l) * (QB + 1) + lane];
                trow[l] = T(0);
            }
            const T ti = lane < bw ? tau[i0 + lane] : T(0);
#pragma unroll
            for (int i = 0; i < QB; i++) {
                const T taui = __shfl_sync(0xffffffffu, ti, i);
                T sum = T(0);
#pragma unroll
                for (int l = 0; l < i; l++) sum += trow[l] * __shfl_sync(0xffffffffu, zc[l], i);
                if (lane < i) trow[i] = -taui * sum;
                else if (lane == i) trow[i] = taui;
            }
            if (lane < bw)
#pragma unroll
                for (int l = 0; l < QB; l++)
                    if (l < bw) Tm[(i0 + lane) + (size_t)(i0 + l) * ldt] = trow[l];
        }
    }
}

// Off-diagonal blocks of the k x k factor T of Q = I - V T V^T over all k reflectors (the
// form in which the one-right-hand-side Orthogonal op applies Q in three passes).  Block
// column j (columns [c0, c0 + bw)) is T[0:c0, j] = -T[0:c0, 0:c0] (V[:, 0:c0]^T V_j) T_j:
// Q_0 ... Q_{j-1} = I - V_A T_A V_A^T merged with Q_j, j ascending.  S = V_A^T V_j is summed
// over the rows >= c0 (V_j is zero above) in 32 x 32 tiles staged in shared memory and
// written into T's block column; M = S T_j replaces it row by row (a warp per row); then
// -T_A M replaces M one 32-row chunk at a time in ascending order (chunk p reads rows >= p
// of M only, so the rows it overwrites are read by no later chunk).  256 threads; sm holds
// 3 x 32 x 33 elements; the diagonal blocks T_j are larft_blocks' (zero below the diagonal).
template <typename T>
__device__ void larft_offdiag(const T* V, int ldv, int rows, int k, T* Tm, int ldt, T* sm) {
    const int tid = threadIdx.x, nth = blockDim.x, lane = tid & 31, w = tid >> 5, nw = nth >> 5;
    constexpr int L = QB + 1;
    T* ta = sm;
    T* tb = sm + QB * L;
    T* tj = sm + 2 * QB * L;
    const int nb = (k + QB - 1) / QB;
    auto vval = [&](int r, int j) -> T { return r > j ? V[r + (size_t)j * ldv] : (r == j ? T(1) : T(0)); };
    for (int jb = 1; jb < nb; jb++) {
        const int c0 = jb * QB, bw = min(QB, k - c0);
        for (int p0 = 0; p0 < c0; p0 += QB) {
            T acc[4] = {T(0), T(0), T(0), T(0)};
            for (int r0 = c0; r0 < rows; r0 += QB) {
                __syncthreads();
                for (int idx = tid; idx < QB * QB; idx += nth) {
                    const int rr = idx % QB, cc = idx / QB, r = r0 + rr;
                    ta[rr * L + cc] = r < rows ? vval(r, p0 + cc) : T(0);
                    tb[rr * L + cc] = (r < rows && cc < bw) ? vval(r, c0 + cc) : T(0);
                }
                __syncthreads();
                for (int rr = 0; rr < QB; rr++) {
                    const T b = tb[rr * L + lane];
                    for (int u = 0; u < 4 && w + nw * u < QB; u++) acc[u] += ta[rr * L + w + nw * u] * b;
                }
            }
            if (lane < bw)
                for (int u = 0; u < 4 && w + nw * u < QB; u++) Tm[(p0 + w + nw * u) + (size_t)(c0 + lane) * ldt] = acc[u];
        }
        for (int idx = tid; idx < QB * QB; idx += nth) {
            const int l = idx % QB, q = idx / QB;
            tj[l * L + q] = (l < bw && q < bw && l <= q) ? Tm[(c0 + l) + (size_t)(c0 + q) * ldt] : T(0);
        }
        __syncthreads();  // S in T's block column, T_j staged
        for (int p = w; p < c0; p += nw) {
            T* sp = Tm + p + (size_t)c0 * ldt;
            const T sv = lane < bw ? sp[(size_t)lane * ldt] : T(0);
            T m = T(0);
            for (int l = 0; l < QB; l++) m += __shfl_sync(0xffffffffu, sv, l) * tj[l * L + lane];
            if (lane < bw) sp[(size_t)lane * ldt] = m;
        }
        for (int p0 = 0; p0 < c0; p0 += QB) {
            T acc[4] = {T(0), T(0), T(0), T(0)};
            for (int l0 = p0; l0 < c0; l0 += QB) {
                __syncthreads();
                for (int idx = tid; idx < QB * QB; idx += nth) {
                    const int pp = idx % QB, ll = idx / QB;
                    ta[ll * L + pp] = p0 + pp <= l0 + ll ? Tm[(p0 + pp) + (size_t)(l0 + ll) * ldt] : T(0);
                    tb[pp * L + ll] = ll < bw ? Tm[(l0 + pp) + (size_t)(c0 + ll) * ldt] : T(0);
                }
                __syncthreads();
                for (int ll = 0; ll < QB; ll++) {
                    const T b = tb[ll * L + lane];
                    for (int u = 0; u < 4 && w + nw * u < QB; u++) acc[u] += ta[ll * L + w + nw * u] * b;
                }
            }
            __syncthreads();  // every thread has read this chunk's rows of M
            if (lane < bw)
                for (int u = 0; u < 4 && w + nw * u < QB; u++)
                    Tm[(p0 + w + nw * u) + (size_t)(c0 + lane) * ldt] = -acc[u];
        }
        __syncthreads();
    }
}

// WY factors of a sparsified cluster's reflectors (for the Orthogonal op of the solve) and
// its tau saved.  One CTA per cluster of the wave.  Reads only the persistent reflector
// store (filled by sparsify_scatter_kernel) and the cluster's own tau slots, so it may
// run beside the QRCP of the next wave.
template <typename T>
__global__ void __launch_bounds__(256) sparsify_wy_kernel(Ctx<T> c, const DSpars* __restrict__ items,
                                                          const T* vstore, const int* __restrict__ rank_in,
                                                          const T* taus_ws, T* taustore, T* tstore, int full_t) {
    if (c.status->not_spd) return;
    const DSpars it = items[blockIdx.x];
    const int rows = c.rows0[it.cluster];
    const int k = rank_in[it.cluster];
    if (k >= rows) return;
    const int ld = c.cap[it.cluster];
    for (int j = threadIdx.x; j < k; j += blockDim.x) taustore[it.tau_off + j] = taus_ws[it.tau_off + j];
    extern __shared__ __align__(16) unsigned char lb_raw[];
    T* sm = reinterpret_cast<T*>(lb_raw);
    larft_blocks(vstore + it.v_off, ld, rows, k, taus_ws + it.tau_off, tstore + it.v_off, ld, sm);
    if (!full_t) return;  // the blocked Orthogonal op needs the diagonal blocks only
    __syncthreads();      // the diagonal blocks written
    larft_offdiag(vstore + it.v_off, ld, rows, k, tstore + it.v_off, ld, sm);
}

// Compressed edges AsnP = triu(R[:k,:]) P^T written back into the cluster's edge blocks,
// the reflectors copied to their persistent store and the cluster's size set to the rank.
// Grid (items, tiles): a CTA copies one 32-column tile of the reflectors (capacity tiles
// first) or of one edge block (then the capacity tiles of every piece).  Column c of Asn
// comes from position ipvt[c] of the QRCP output.  Every CTA reads the cluster's own size
// from the level snapshot (rows0), so the first one can set csize right away.
template <typename T>
__global__ void __launch_bounds__(256) sparsify_scatter_kernel(Ctx<T> c, const DSpars* __restrict__ items,
                                                               const DAsn* __restrict__ pieces, const T* ws,
                                                               const int* __restrict__ ipvt_ws,
                                                               const int* __restrict__ rank_in, T* vstore) {
    pdl_wait_and_release();
    __shared__ T tile[32][33];
    __shared__ int qs[32];
    if (c.status->not_spd) return;
    const DSpars it = items[blockIdx.x];
    const int rows = c.rows0[it.cluster];
    const int k = rank_in[it.cluster];
    if (k >= rows) return;
    if (blockIdx.y == 0 && threadIdx.x == 0) c.csize[it.cluster] = k;
    const int ld = c.cap[it.cluster];
    const T* A = ws + it.ws_off;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int t = blockIdx.y;
    const int nvt = (ld + 31) / 32;
    if (t < nvt) {
        T* V = vstore + it.v_off;
        for (int jj = w; jj < 32; jj += nw) {
            const int j = 32 * t + jj;
            if (j >= k) break;
            for (int r = lane; r < rows; r += 32) V[r + (size_t)j * ld] = A[r + (size_t)j * ld];
        }
        return;
    }
    t -= nvt;
    int col = 0, p = 0;
    for (; p < it.count; p++) {
        const int nbr = pieces[it.first + p].nbr;
        const int nt = (c.cap[nbr] + 31) / 32;
        if (t < nt) break;
        t -= nt;
        col += c.csize[nbr];
    }
    if (p >= it.count) return;
    const DAsn pc = pieces[it.first + p];
    const int n = c.csize[pc.nbr];
    const int j0 = 32 * t;
    if (j0 >= n) return;
    const int jw = min(32, n - j0);
    const int* ipvt = ipvt_ws + it.col_off + col + j0;
    T* B = bptr(c, pc.block);
    const int bld = c.blk[pc.block].ld;
    if (!pc.transposed) {
        for (int jj = w; jj < jw; jj += nw) {
            const int q = ipvt[jj];
            const T* src = A + (size_t)q * ld;
            T* dst = B + (size_t)(j0 + jj) * bld;
            for (int i = lane; i < k; i += 32) dst[i] = i <= q ? src[i] : T(0);
        }
    } else {
        if (threadIdx.x < jw) qs[threadIdx.x] = ipvt[threadIdx.x];
        __syncthreads();
        for (int i0 = 0; i0 < k; i0 += 32) {
            const int i = i0 + lane;
            for (int jj = w; jj < jw; jj += nw) {
                const int q = qs[jj];
                tile[jj][lane] = (i < k && i <= q) ? A[i + (size_t)q * ld] : T(0);
            }
            __syncthreads();
            for (int ii = w; ii < 32 && i0 + ii < k; ii += nw)
                if (lane < jw) B[(j0 + lane) + (size_t)(i0 + ii) * bld] = tile[lane][ii];
            __syncthreads();
        }
    }
}

// ------------------------------------------------------------------------------------
// Merge (tree.cpp:1106-1184)
// ------------------------------------------------------------------------------------
__global__ void merge_sizes_kernel(int* csize, int* rows0, int* cpos, const int* __restrict__ parents, int np,
                                   const int* __restrict__ child_ptr, const int* __restrict__ child_idx) {
    pdl_wait_and_release();
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

constexpr int MT = 64;  // a 64 x 64 tile per CTA: sixteen elements per thread

template <typename T>
__global__ void merge_copy_kernel(Ctx<T> c, const DMerge* __restrict__ items, const DTile* __restrict__ tiles,
                                  int ntiles, const int* __restrict__ cpos) {
    pdl_wait_and_release();
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

// Assembly of the level-0 blocks on the device: blocks[map[k]] = vals[k] (block2dense,
// util.cpp:454-486, as a scatter; the blocks are zeroed first).
template <typename T>
__global__ void assemble_scatter_kernel(const double* __restrict__ vals, const long long* __restrict__ map,
                                        long long n, T* blocks) {
    long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k >= n) return;
    const long long d = map[k];
    if (d >= 0) blocks[d] = (T)vals[k];
}

__global__ void scatter_f64_kernel(const double* __restrict__ src, const int* __restrict__ map, long long n,
                                   double* dst) {
    long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k < n && map[k] >= 0) dst[map[k]] = src[k];
}

// out[k] = -lam[rows[k]] * x[cols[k]]: the adjoint -lambda x^T restricted to the stored
// entries of A (one entry per thread; the gathers of lam and x hit L2 for stencil patterns)
__global__ void pattern_outer_kernel(long long nnz, const int* __restrict__ rows, const int* __restrict__ cols,
                                     const double* __restrict__ lam, const double* __restrict__ x,
                                     double* __restrict__ out) {
    long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k < nnz) out[k] = -lam[rows[k]] * x[cols[k]];
}

// LoRaSp: the new pivot of a scaled cluster, a stored identity (the block is zero from the
// factorization's start); one CTA per cluster
template <typename T>
__global__ void identity_kernel(Ctx<T> c, const int* __restrict__ blocks, const int* __restrict__ clusters) {
    const int n = c.csize[clusters[blockIdx.x]];
    T* B = bptr(c, blocks[blockIdx.x]);
    const int ld = c.blk[blocks[blockIdx.x]].ld;
    for (int i = threadIdx.x; i < n; i += blockDim.x) B[i + (size_t)i * ld] = T(1);
}

__global__ void snapshot_kernel(const int* csize, int* rows0, const int* __restrict__ clusters, int n) {
    pdl_wait_and_release();
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

// ScalingPLUQ of the solve (operations.cpp:112-127, q = identity for PLU): forward
// x_s <- L_s^{-1} P^T x_s, backward x_s <- U_s^{-1} x_s, as products with the inverse
// block (consecutive threads read consecutive rows of one of its columns).  One CTA per
// (cluster, right-hand side); x_s is staged in shared memory.
template <typename T>
__global__ void __launch_bounds__(256) lu_apply_kernel(Ctx<T> c, XCtx<T> X, const int* __restrict__ clusters,
                                                      const int* __restrict__ invs, int count,
                                                      const int* __restrict__ perm_store,
                                                      const long long* __restrict__ poff, int fwd) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* xs = reinterpret_cast<T*>(smem_raw);
    const int item = blockIdx.x, r = blockIdx.y;
    if (item >= count) return;
    const int cid = clusters[item];
    const int n = c.rows0[cid];  // the size when the pivot was factored (before sparsification)
    if (n == 0) return;
    T* x = X.xs + X.xoff[cid] + (long long)r * X.xld;
    const T* W = bptr(c, invs[item]);
    const int wld = c.blk[invs[item]].ld;
    const int* perm = perm_store + poff[cid];
    for (int i = threadIdx.x; i < n; i += blockDim.x) xs[i] = fwd ? x[perm[i]] : x[i];
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        T s0 = 0, s1 = 0;
        if (fwd) {
            int k = 0;
            for (; k + 1 < i; k += 2) {
                s0 += W[i + (size_t)k * wld] * xs[k];
                s1 += W[i + (size_t)(k + 1) * wld] * xs[k + 1];
            }
            for (; k < i; k++) s0 += W[i + (size_t)k * wld] * xs[k];
            s0 += (T)fabs(W[i + (size_t)i * wld]) * xs[i];
        } else {
            int k = i;
            for (; k + 1 < n; k += 2) {
                s0 += W[i + (size_t)k * wld] * xs[k];
                s1 += W[i + (size_t)(k + 1) * wld] * xs[k + 1];
            }
            for (; k < n; k++) s0 += W[i + (size_t)k * wld] * xs[k];
        }
        x[i] = s0 + s1;
    }
}

// LDLT solve steps (operations.cpp:128-142, 44-53):
// perm_x_kernel: x_s <- P^T x_s (fwd, before L_s^{-1}) or x_s <- P x_s (bwd, after L_s^{-T});
// sign_x_kernel: the diag phase, x_s <- D^{-1} x_s = s .* x_s;
// split_x_kernel: the Split op, x_sib <- x_c[k:r] (fwd) or x_c[k:r] <- x_sib (bwd).
// One CTA per (cluster, right-hand side); sizes rows0 (the size when the op was recorded).
template <typename T>
__global__ void perm_x_kernel(Ctx<T> c, XCtx<T> X, const int* __restrict__ clusters, int count,
                              const int* __restrict__ perm_store, const long long* __restrict__ poff, int fwd) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* t = reinterpret_cast<T*>(smem_raw);
    const int item = blockIdx.x, r = blockIdx.y;
    if (item >= count) return;
    const int cid = clusters[item];
    const int n = c.rows0[cid];
    T* x = X.xs + X.xoff[cid] + (long long)r * X.xld;
    const int* perm = perm_store + poff[cid];
    for (int i = threadIdx.x; i < n; i += blockDim.x) t[i] = x[i];
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        if (fwd) x[i] = t[perm[i]];
        else x[perm[i]] = t[i];
    }
}

template <typename T>
__global__ void sign_x_kernel(Ctx<T> c, XCtx<T> X, const int* __restrict__ clusters, int count,
                              const T* __restrict__ sign_store, const long long* __restrict__ poff) {
    const int item = blockIdx.x, r = blockIdx.y;
    if (item >= count) return;
    const int cid = clusters[item];
    const int n = c.rows0[cid];
    T* x = X.xs + X.xoff[cid] + (long long)r * X.xld;
    const T* s = sign_store + poff[cid];
    for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] *= s[i];
}

template <typename T>
__global__ void split_x_kernel(Ctx<T> c, XCtx<T> X, const int* __restrict__ owners, const int* __restrict__ sibs,
                               int count, int fwd) {
    const int item = blockIdx.x, r = blockIdx.y;
    if (item >= count) return;
    const int cl = owners[item], sb = sibs[item];
    const int k = c.csize[cl], m = c.csize[sb];
    T* xc = X.xs + X.xoff[cl] + (long long)r * X.xld + k;
    T* xsb = X.xs + X.xoff[sb] + (long long)r * X.xld;
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        if (fwd) xsb[i] = xc[i];
        else xc[i] = xsb[i];
    }
}

// b = P^T x (natural -> permuted leaf slots), FP64 in, T out
template <typename T>
__global__ void perm_in_kernel(const double* __restrict__ x, int ldx, XCtx<T> X, const int* __restrict__ perm,
                               const long long* __restrict__ slot, int n) {
    pdl_wait_and_release();
    long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k >= (long long)n * X.nrhs) return;
    int p = (int)(k % n), r = (int)(k / n);
    X.xs[slot[p] + r * X.xld] = (T)x[perm[p] + (size_t)r * ldx];
}

template <typename T>
__global__ void perm_out_kernel(double* __restrict__ x, int ldx, XCtx<T> X, const int* __restrict__ perm,
                                const long long* __restrict__ slot, int n) {
    pdl_wait_and_release();
    long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k >= (long long)n * X.nrhs) return;
    int p = (int)(k % n), r = (int)(k / n);
    x[perm[p] + (size_t)r * ldx] = (double)X.xs[slot[p] + r * X.xld];
}

// Triangular products of the solve (ScalingLLT, operations.cpp:97-103): forward
// x_c <- L_c^{-1} x_c, backward x_c <- L_c^{-T} x_c.  L^{-1} is stored transposed in the
// strictly upper triangle of the pivot block (row i of L^{-1} = column i of the block),
// its diagonal as 1 / L_ii.  Work list: (cluster, row tile).  A cluster of at most
// 2*TV_ROWS rows is one tile, computed in place by one CTA; a larger one is cut into
// TV_ROWS-row tiles whose CTAs write their rows to the scratch copy of the solve vectors;
// the last CTA of the cluster to finish (atomic counter, reset by that CTA) copies the
// rows back.  Forward: warp per row, lanes over the columns; backward: lanes over the
// rows, warps over the columns, partial sums added in a fixed order.  All right-hand
// sides in one CTA.  Shared memory: the staged x range + 8 x 2*TV_ROWS partial sums.
constexpr int TV_ROWS = 32;
constexpr int TV_THREADS = 256;

template <typename T>
__device__ __forceinline__ void trsv4_body(Ctx<T> c, XCtx<T> X, const int* __restrict__ clusters,
                                           const int* __restrict__ lblocks, const int2* __restrict__ tiles,
                                           int trans, T* tmp, int* counters, int bid) {
    const int2 tl = tiles[bid];
    const int item = tl.x, tile = tl.y;
    const int cl = clusters[item];
    const int n = c.rows0[cl];
    const int nt = n <= 2 * TV_ROWS ? 1 : (n + TV_ROWS - 1) / TV_ROWS;
    if (n == 0 || tile >= nt) return;
    const int r0 = nt == 1 ? 0 : tile * TV_ROWS, r1 = nt == 1 ? n : min(n, r0 + TV_ROWS);
    const T* L = bptr(c, lblocks[item]);
    const int ld = c.blk[lblocks[item]].ld;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int NW = TV_THREADS / 32;
    T* part = reinterpret_cast<T*>(smem_raw);  // NW x 2*TV_ROWS
    T* xs = part + NW * 2 * TV_ROWS;            // x[lo, hi)
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int lo = trans ? r0 : 0, hi = trans ? n : r1;
    for (int rhs = 0; rhs < X.nrhs; rhs++) {
        const T* x = X.xs + X.xoff[cl] + (size_t)rhs * X.xld;
        T* y = (nt == 1 ? X.xs : tmp) + X.xoff[cl] + (size_t)rhs * X.xld;
        __syncthreads();
        for (int k = lo + threadIdx.x; k < hi; k += TV_THREADS) xs[k - lo] = x[k];
        __syncthreads();
        if (!trans) {
            for (int row = r0 + w; row < r1; row += NW) {
                const T* lrow = L + (size_t)row * ld;
                T a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                int k = lane;
                for (; k + 7 * 32 < row; k += 8 * 32) {
#pragma unroll
                    for (int u = 0; u < 8; u++) a[u] += lrow[k + 32 * u] * xs[k + 32 * u];
                }
                for (; k < row; k += 32) a[0] += lrow[k] * xs[k];
                const T s = warp_sum(((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7])));
                if (lane == 0) y[row] = s + xs[row] / L[row + (size_t)row * ld];
            }
        } else {
            const int nr = r1 - r0;
            for (int rb = 0; rb < nr; rb += 32) {
                const int row = r0 + rb + lane;
                const bool live = rb + lane < nr;
                T a[4] = {0, 0, 0, 0};
                int k = r0 + 1 + w;
                for (; k + 3 * NW < n; k += 4 * NW) {
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const int kk = k + u * NW;
                        if (live && row < kk) a[u] += L[row + (size_t)kk * ld] * xs[kk - lo];
                    }
                }
                for (; k < n; k += NW)
                    if (live && row < k) a[0] += L[row + (size_t)k * ld] * xs[k - lo];
                part[w * 2 * TV_ROWS + rb + lane] = (a[0] + a[1]) + (a[2] + a[3]);
            }
            __syncthreads();
            for (int q = threadIdx.x; q < nr; q += TV_THREADS) {
                T s = 0;
                for (int ww = 0; ww < NW; ww++) s += part[ww * 2 * TV_ROWS + q];
                const int row = r0 + q;
                y[row] = s + xs[row - lo] / L[row + (size_t)row * ld];
            }
        }
    }
    if (nt == 1) return;
    // the last tile of the cluster copies the rows of every tile back
    __threadfence();
    __syncthreads();
    __shared__ int last;
    if (threadIdx.x == 0) last = atomicAdd(&counters[cl], 1) == nt - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    for (int rhs = 0; rhs < X.nrhs; rhs++) {
        const size_t off = X.xoff[cl] + (size_t)rhs * X.xld;
        for (int k = threadIdx.x; k < n; k += TV_THREADS) X.xs[off + k] = __ldcg(tmp + off + k);
    }
    if (threadIdx.x == 0) counters[cl] = 0;
}

template <typename T>
__global__ void __launch_bounds__(TV_THREADS) trsv4_kernel(Ctx<T> c, XCtx<T> X, const int* __restrict__ clusters,
                                                          const int* __restrict__ lblocks,
                                                          const int2* __restrict__ tiles, int trans, T* tmp,
                                                          int* counters) {
    pdl_wait_and_release();
    trsv4_body<T>(c, X, clusters, lblocks, tiles, trans, tmp, counters, blockIdx.x);
}

// The triangular products (as trsv4_kernel) of clusters of at most 64 rows, one warp per
// cluster, eight clusters per CTA: x in registers (rows lane and lane + 32), every x_k
// reaches the lanes by shuffle.  Forward y_i = x_i / L_ii + sum_{k<i} L^{-1}[i][k] x_k with
// lane i walking row i of L^{-1} (column i of the block, contiguous); backward
// y_k = x_k / L_kk + sum_{i>k} L^{-1}[i][k] x_i with consecutive lanes on consecutive
// entries of each column (coalesced).  In place: the warp holds all of x before it writes.
constexpr int TS_WARPS = 8;
template <typename T>
__device__ __forceinline__ void trsv_small_body(Ctx<T> c, XCtx<T> X, const int* __restrict__ clusters,
                                                const int* __restrict__ lblocks, const int* __restrict__ idx,
                                                int count, int trans, int bid) {
    const int lane = threadIdx.x & 31;
    const int item = bid * TS_WARPS + (threadIdx.x >> 5);
    if (item >= count) return;
    const int k = idx[item];
    const int cl = clusters[k];
    const int n = c.rows0[cl];
    if (n == 0) return;
    const T* __restrict__ L = bptr(c, lblocks[k]);
    const int ld = c.blk[lblocks[k]].ld;
    const int ia = lane, ib = lane + 32;
    const T da = ia < n ? L[ia + (size_t)ia * ld] : T(1);
    const T db = ib < n ? L[ib + (size_t)ib * ld] : T(1);
    for (int rhs = 0; rhs < X.nrhs; rhs++) {
        T* x = X.xs + X.xoff[cl] + (size_t)rhs * X.xld;
        const T xa = ia < n ? x[ia] : T(0);
        const T xb = ib < n ? x[ib] : T(0);
        T sa0 = xa / da, sa1 = T(0), sb0 = xb / db, sb1 = T(0);
        if (!trans) {
            // row i of L^{-1} is read only for rows of the cluster (i < n) and only left of
            // its diagonal (q < i); eight columns at a time, their loads issued together
            const int ea = ia < n ? ia : 0, eb = ib < n ? ib : 0;
            const T* la = L + (size_t)ea * ld;
            const T* lb = L + (size_t)eb * ld;
            for (int q0 = 0; q0 < n; q0 += 8) {
                T va[8], vb[8];
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    va[u] = q0 + u < ea ? la[q0 + u] : T(0);
                    vb[u] = q0 + u < eb ? lb[q0 + u] : T(0);
                }
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    const int q = q0 + u;
                    const T xq = __shfl_sync(0xffffffffu, q < 32 ? xa : xb, q & 31);
                    if (u & 1) {
                        sa1 += va[u] * xq;
                        sb1 += vb[u] * xq;
                    } else {
                        sa0 += va[u] * xq;
                        sb0 += vb[u] * xq;
                    }
                }
            }
        } else {
            // y_k += sum_{q>k} L^{-1}[q][k] x_q: column q of the block, consecutive lanes on
            // consecutive entries; eight columns at a time
            for (int q0 = 1; q0 < n; q0 += 8) {
                T va[8], vb[8];
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    const int q = q0 + u;
                    const T* lq = L + (size_t)(q < n ? q : 0) * ld;
                    va[u] = (q < n && ia < q) ? lq[ia] : T(0);
                    vb[u] = (q < n && ib < q) ? lq[ib] : T(0);
                }
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    const int q = q0 + u;
                    const T xq = __shfl_sync(0xffffffffu, q < 32 ? xa : xb, q & 31);
                    if (u & 1) {
                        sa1 += va[u] * xq;
                        sb1 += vb[u] * xq;
                    } else {
                        sa0 += va[u] * xq;
                        sb0 += vb[u] * xq;
                    }
                }
            }
        }
        if (ia < n) x[ia] = sa0 + sa1;
        if (ib < n) x[ib] = sb0 + sb1;
    }
}

template <typename T>
__global__ void __launch_bounds__(32 * TS_WARPS) trsv_small_kernel(Ctx<T> c, XCtx<T> X,
                                                                   const int* __restrict__ clusters,
                                                                   const int* __restrict__ lblocks,
                                                                   const int* __restrict__ idx, int count, int trans) {
    pdl_wait_and_release();
    trsv_small_body<T>(c, X, clusters, lblocks, idx, count, trans, blockIdx.x);
}

// Both of a phase's triangular products in one launch: the first nsb CTAs take the small
// clusters a warp each (trsv_small_body), the others the row tiles of the larger ones
// (trsv4_body).  The two sets of clusters are disjoint, so the halves need no order
// between them, and the phase costs one launch instead of two.
static_assert(32 * TS_WARPS == TV_THREADS, "one block shape for both halves");
template <typename T>
__global__ void __launch_bounds__(TV_THREADS) trsv_fused_kernel(Ctx<T> c, XCtx<T> X, const int* __restrict__ clusters,
                                                               const int* __restrict__ lblocks,
                                                               const int* __restrict__ idx, int count, int nsb,
                                                               const int2* __restrict__ tiles, int trans, T* tmp,
                                                               int* counters) {
    pdl_wait_and_release();
    if ((int)blockIdx.x < nsb) trsv_small_body<T>(c, X, clusters, lblocks, idx, count, trans, blockIdx.x);
    else trsv4_body<T>(c, X, clusters, lblocks, tiles, trans, tmp, counters, (int)blockIdx.x - nsb);
}

// One Gemm op's operands as the solve kernels use them: the factor block, the solve
// vector it multiplies, its length and the LDLT signs.
template <typename T>
struct GemmMeta {
    const T* A;
    const T* x;
    const T* sg;
    int ld, n, kind;
};
constexpr int GM_CHUNK = 64;

// Forward Gemm ops grouped by neighbour n (operations.cpp:55-93): x_n -= sum over the
// group's ops of A_ns x_s (GemmSymmOut) or A_sn^T x_s (GemmSymmIn), in op order.  One
// block per (group, 64 rows of x_n); 4 threads per row split the columns, partial sums
// reduced in a fixed order.
constexpr int GF_ROWS = 64;

// LDLT path: signs != nullptr weights x_self by the signs of self (A D x_s,
// operations.cpp:55-83); sib_mode: the neighbour is a sparsified cluster whose size is now
// csize (the op of a sibling, recorded after the split).  An op kind with bit 16 set says
// the same for its own neighbour (LoRaSp siblings, whose neighbours may or may not have
// been sparsified before them).
template <typename T>
__global__ void __launch_bounds__(256) gemm_fwd2_kernel(Ctx<T> c, XCtx<T> X, const DGroup* __restrict__ groups,
                                                        const DGemmOp* __restrict__ ops, const DTile* __restrict__ tiles,
                                                        int ntiles, int rhs_stride, const T* __restrict__ signs = nullptr,
                                                        const long long* __restrict__ soff = nullptr,
                                                        int sib_mode = 0) {
    pdl_wait_and_release();
    const int t = blockIdx.x % ntiles;
    const int r = blockIdx.x / ntiles;
    const DGroup G = groups[tiles[t].item];
    const int nb = G.key;
    const int nn = (sib_mode || (ops[G.first].kind & 16)) ? c.csize[nb] : c.rows0[nb];
    const int i0 = tiles[t].tile_i * GF_ROWS;
    if (i0 >= nn) return;
    (void)rhs_stride;
    __shared__ T part[4][GF_ROWS];
    __shared__ T racc[GF_ROWS];  // the GemmSymmIn products, a warp per row
    T* xn = X.xs + X.xoff[nb] + r * X.xld;
    const int li = threadIdx.x % GF_ROWS, sp = threadIdx.x / GF_ROWS;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    constexpr int RPW = GF_ROWS / 8;  // rows per warp in the GemmSymmIn products
    const int i = i0 + li;
    if (threadIdx.x < GF_ROWS) racc[threadIdx.x] = T(0);
    // the ops' operands, GM_CHUNK at a time, looked up by one thread each (the lookups are
    // chains of dependent loads; done in parallel they cost one chain per chunk, not per op)
    __shared__ GemmMeta<T> meta[GM_CHUNK];
    T acc = 0;
    for (int o0 = 0; o0 < G.count; o0 += GM_CHUNK) {
        const int cnt = min(GM_CHUNK, G.count - o0);
        __syncthreads();
        if (threadIdx.x < cnt) {
            const DGemmOp op = ops[G.first + o0 + threadIdx.x];
            GemmMeta<T> m;
            m.n = c.csize[op.self];
            m.x = X.xs + X.xoff[op.self] + r * X.xld;
            m.A = bptr(c, op.block);
            m.ld = c.blk[op.block].ld;
            m.sg = signs ? signs + soff[op.self] : nullptr;
            m.kind = op.kind & 15;
            meta[threadIdx.x] = m;
        }
        __syncthreads();
        // two ops per pass: the second op's loads issue while the first's are in flight
#pragma unroll 2
        for (int o = 0; o < cnt; o++) {
            const GemmMeta<T> m = meta[o];
            const int ns = m.n;
            const T* xs = m.x;
            const T* A = m.A;
            const int ld = m.ld;
            const T* sg = m.sg;
            const int kind = m.kind;
            if (kind == 1) {
                // A_ns x_s: a thread per row (consecutive rows read consecutive entries)
                if (i < nn) {
                    T s0 = 0, s1 = 0, s2 = 0, s3 = 0;
                    int j = sp;
                    if (sg) {
                        for (; j < ns; j += 4) s0 += A[i + (size_t)j * ld] * (sg[j] * xs[j]);
                    } else {
                        for (; j + 12 < ns; j += 16) {
                            s0 += A[i + (size_t)j * ld] * xs[j];
                            s1 += A[i + (size_t)(j + 4) * ld] * xs[j + 4];
                            s2 += A[i + (size_t)(j + 8) * ld] * xs[j + 8];
                            s3 += A[i + (size_t)(j + 12) * ld] * xs[j + 12];
                        }
                        for (; j < ns; j += 4) s0 += A[i + (size_t)j * ld] * xs[j];
                    }
                    acc += (s0 + s1) + (s2 + s3);
                }
            } else {
                // A_sn^T x_s: row i is column i of A_sn; a warp per RPW rows, lanes over j
                // (consecutive lanes read consecutive entries), the rows' sums in parallel
                T sr[RPW];
#pragma unroll
                for (int u = 0; u < RPW; u++) sr[u] = T(0);
                for (int j = lane; j < ns; j += 32) {
                    const T xj = sg ? sg[j] * xs[j] : xs[j];
#pragma unroll
                    for (int u = 0; u < RPW; u++) {
                        const int ii = i0 + wid * RPW + u;
                        if (ii < nn) sr[u] += A[j + (size_t)ii * ld] * xj;
                    }
                }
#pragma unroll
                for (int u = 0; u < RPW; u++) {
                    const T v = warp_sum(sr[u]);
                    if (lane == 0) racc[wid * RPW + u] += v;
                }
            }
        }
    }
    part[sp][li] = acc;
    __syncthreads();
    if (sp == 0 && i < nn) xn[i] -= ((part[0][li] + part[1][li]) + (part[2][li] + part[3][li])) + racc[li];
}

// Backward Gemm ops grouped by eliminated cluster s: x_s -= sum of A_ns^T x_n
// (GemmSymmOut) or A_sn x_n (GemmSymmIn), ops in reverse recording order.  One block per
// (s, 32 entries of x_s): a warp per entry where the entry's terms are contiguous
// (A_ns^T), a thread per entry with eight column slices where they are strided (A_sn).
constexpr int GB_ROWS = 32;

template <typename T>
__global__ void __launch_bounds__(256) gemm_bwd2_kernel(Ctx<T> c, XCtx<T> X, const DGroup* __restrict__ groups,
                                                        const DGemmOp* __restrict__ ops, const DTile* __restrict__ tiles,
                                                        int ntiles, const T* __restrict__ signs = nullptr,
                                                        const long long* __restrict__ soff = nullptr,
                                                        int sib_mode = 0) {
    pdl_wait_and_release();
    const int t = blockIdx.x % ntiles;
    const int r = blockIdx.x / ntiles;
    const DGroup G = groups[tiles[t].item];
    const int sc = G.key;
    const int ns = c.csize[sc];
    const int i0 = tiles[t].tile_i * GB_ROWS;
    if (i0 >= ns) return;
    T* xs = X.xs + X.xoff[sc] + r * X.xld;
    __shared__ T wacc[GB_ROWS];      // the A_ns^T terms, a warp per entry
    __shared__ T part[8][GB_ROWS];   // the A_sn terms, eight column slices
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int li = threadIdx.x % GB_ROWS, sp = threadIdx.x / GB_ROWS;  // 8 slices of 256 threads
    T pacc = 0;
    T wsum[GB_ROWS / 8];
#pragma unroll
    for (int u = 0; u < GB_ROWS / 8; u++) wsum[u] = T(0);
    __shared__ GemmMeta<T> meta[GM_CHUNK];  // as in gemm_fwd2_kernel
    for (int o0 = 0; o0 < G.count; o0 += GM_CHUNK) {
        const int cnt = min(GM_CHUNK, G.count - o0);
        __syncthreads();
        if (threadIdx.x < cnt) {
            const DGemmOp op = ops[G.first + o0 + threadIdx.x];
            GemmMeta<T> m;
            m.n = (sib_mode || (op.kind & 16)) ? c.csize[op.nbr] : c.rows0[op.nbr];
            m.x = X.xs + X.xoff[op.nbr] + r * X.xld;
            m.A = bptr(c, op.block);
            m.ld = c.blk[op.block].ld;
            m.sg = nullptr;
            m.kind = op.kind & 15;
            meta[threadIdx.x] = m;
        }
        __syncthreads();
        // two ops per pass: the second op's loads issue while the first's are in flight
#pragma unroll 2
        for (int o = 0; o < cnt; o++) {
            const GemmMeta<T> m = meta[o];
            const int nn = m.n;
            const T* xn = m.x;
            const T* A = m.A;
            const int ld = m.ld;
            if (m.kind == 1) {
                // A_ns^T x_n: entry i is column i of A_ns; the warp's entries side by side in
                // one pass over j (their loads issue together)
                const T* au[GB_ROWS / 8];
                bool live[GB_ROWS / 8];
#pragma unroll
                for (int u = 0; u < GB_ROWS / 8; u++) {
                    const int ii = w + nw * u;
                    live[u] = ii < GB_ROWS && i0 + ii < ns;
                    au[u] = A + (size_t)(live[u] ? i0 + ii : 0) * ld;
                }
                for (int j = lane; j < nn; j += 32) {
                    const T xj = xn[j];
#pragma unroll
                    for (int u = 0; u < GB_ROWS / 8; u++)
                        if (live[u]) wsum[u] += au[u][j] * xj;
                }
            } else {
                // A_sn x_n: a thread per entry, column slices j = sp (mod 8), four loads in
                // flight
                const int i = i0 + li;
                if (i < ns) {
                    T s0 = 0, s1 = 0, s2 = 0, s3 = 0;
                    int j = sp;
                    for (; j + 24 < nn; j += 32) {
                        s0 += A[i + (size_t)j * ld] * xn[j];
                        s1 += A[i + (size_t)(j + 8) * ld] * xn[j + 8];
                        s2 += A[i + (size_t)(j + 16) * ld] * xn[j + 16];
                        s3 += A[i + (size_t)(j + 24) * ld] * xn[j + 24];
                    }
                    for (; j < nn; j += 8) s0 += A[i + (size_t)j * ld] * xn[j];
                    pacc += (s0 + s1) + (s2 + s3);
                }
            }
        }
    }
#pragma unroll
    for (int u = 0; u < GB_ROWS / 8; u++) {
        const T v = warp_sum(wsum[u]);
        const int ii = w + nw * u;
        if (lane == 0 && ii < GB_ROWS) wacc[ii] = v;
    }
    part[sp][li] = pacc;
    __syncthreads();
    if (threadIdx.x < GB_ROWS) {
        const int i = i0 + threadIdx.x;
        if (i < ns) {
            T acc = wacc[threadIdx.x];
            for (int q = 0; q < 8; q++) acc += part[q][threadIdx.x];
            xs[i] -= signs ? signs[soff[sc] + i] * acc : acc;  // LDLT: D (A^T x_n)
        }
    }
}

// Orthogonal op of the solve with the blocked WY form: fwd x <- Q^T x applies
// Q_b^T = I - V_b T_b^T V_b^T for b = 0, 1, ...; bwd x <- Q x applies Q_b for b = nb-1 ... 0
// (operations.cpp:153-158).  Three barriers per block of 32 reflectors.  Where the shared
// memory holds them (staged), each block's reflectors (rows >= the block's first) and its
// T factor are first copied there by the whole CTA with coalesced loads, all in flight at
// once, so that the three phases read shared memory instead of chains of L2 loads.
template <typename T>
__global__ void __launch_bounds__(512) ortho_wyb_kernel(Ctx<T> c, XCtx<T> X, const DOrtho* __restrict__ items,
                                                        int count, const T* vstore, const T* tstore, int trans,
                                                        int smem_elems) {
    pdl_wait_and_release();
    const int item = blockIdx.x % count;
    const int r = blockIdx.x / count;
    const DOrtho it = items[item];
    const int rows = c.rows0[it.cluster];
    const int k = c.csize[it.cluster];
    if (k >= rows || k == 0) return;
    const int ld = c.cap[it.cluster];
    const T* V = vstore + it.v_off;
    const T* Tm = tstore + it.v_off;
    T* x = X.xs + X.xoff[it.cluster] + r * X.xld;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* xs = reinterpret_cast<T*>(smem_raw);  // rows
    T* tb = xs + rows;                        // T_b, 32 x 33
    T* vb = tb + QB * (QB + 1);               // V_b rows [i0, rows), column i at vb + i * (rows - i0)
    const bool staged = (long long)rows + QB * (QB + 1) + (long long)QB * rows <= smem_elems;
    __shared__ T wv[QB], yv[QB];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int i = threadIdx.x; i < rows; i += blockDim.x) xs[i] = x[i];
    __syncthreads();
    const int nb = (k + QB - 1) / QB;
    for (int q = 0; q < nb; q++) {
        const int b = trans ? q : nb - 1 - q;
        const int i0 = b * QB, bw = min(QB, k - i0);
        const int h = rows - i0;
        if (staged) {
            for (int idx = threadIdx.x; idx < h * bw; idx += blockDim.x) {
                const int rr = idx % h, i = idx / h;
                vb[idx] = V[(i0 + rr) + (size_t)(i0 + i) * ld];
            }
            for (int idx = threadIdx.x; idx < bw * bw; idx += blockDim.x) {
                const int jj = idx % bw, i = idx / bw;
                tb[jj + i * (QB + 1)] = Tm[(i0 + jj) + (size_t)(i0 + i) * ld];
            }
            __syncthreads();
        }
        // w = V_b^T x
        for (int i = w; i < bw; i += nw) {
            T s = 0;
            if (staged) {
                const T* vi = vb + (size_t)i * h;
                for (int rr = i + 1 + lane; rr < h; rr += 32) s += vi[rr] * xs[i0 + rr];
            } else {
                const T* vi = V + (size_t)(i0 + i) * ld;
                for (int rr = i0 + i + 1 + lane; rr < rows; rr += 32) s += vi[rr] * xs[rr];
            }
            s = warp_sum(s);
            if (lane == 0) wv[i] = xs[i0 + i] + s;
        }
        __syncthreads();
        // y = T_b^T w (fwd) or T_b w (bwd)
        if (threadIdx.x < bw) {
            const int i = threadIdx.x;
            T s = 0;
            if (trans) {
                for (int j = 0; j <= i; j++)
                    s += (staged ? tb[j + i * (QB + 1)] : Tm[(i0 + j) + (size_t)(i0 + i) * ld]) * wv[j];
            } else {
                for (int j = i; j < bw; j++)
                    s += (staged ? tb[i + j * (QB + 1)] : Tm[(i0 + i) + (size_t)(i0 + j) * ld]) * wv[j];
            }
            yv[i] = s;
        }
        __syncthreads();
        // x -= V_b y
        for (int rr = i0 + threadIdx.x; rr < rows; rr += blockDim.x) {
            const int imax = min(rr - i0, bw - 1);
            T s = 0;
            for (int i = 0; i <= imax; i++)
                s += (i0 + i == rr ? T(1) : (staged ? vb[(rr - i0) + (size_t)i * h] : V[rr + (size_t)(i0 + i) * ld])) * yv[i];
            xs[rr] -= s;
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < rows; i += blockDim.x) x[i] = xs[i];
}

// Orthogonal op with the whole compact WY factor (T: k x k upper triangular, off-diagonal
// blocks from larft_offdiag): fwd x <- Q^T x = x - V T^T V^T x, bwd x <- Q x = x - V T V^T x
// (operations.cpp:153-158) in three passes and two barriers whatever k: w = V^T x (a warp
// per four reflectors, lanes down their columns), y = T^T w (a warp per four entries, lanes
// down T's columns) or T w (a thread per entry, consecutive threads on consecutive rows of
// T), then x -= V y (a thread per row, consecutive threads on consecutive rows of V).  Every
// factor read is coalesced, and each thread keeps four to eight independent loads in
// flight (the passes are bound by load latency, not bandwidth); V is read twice and T
// once, straight from global memory.  One CTA per (cluster, right-hand side); shared
// memory: x (rows), w and y (k each).
template <typename T, int NT>
__global__ void __launch_bounds__(NT) ortho_full_kernel(Ctx<T> c, XCtx<T> X, const DOrtho* __restrict__ items,
                                                        int count, const T* __restrict__ vstore,
                                                        const T* __restrict__ tstore, int trans) {
    pdl_wait_and_release();
    const int item = blockIdx.x % count;
    const int r = blockIdx.x / count;
    const DOrtho it = items[item];
    const int rows = c.rows0[it.cluster];
    const int k = c.csize[it.cluster];
    if (k >= rows || k == 0) return;
    const int ld = c.cap[it.cluster];
    const T* __restrict__ V = vstore + it.v_off;
    const T* __restrict__ Tm = tstore + it.v_off;
    T* x = X.xs + X.xoff[it.cluster] + (size_t)r * X.xld;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* xs = reinterpret_cast<T*>(smem_raw);
    T* wv = xs + rows;
    T* yv = wv + k;
    constexpr int NW = NT / 32;
    constexpr int C4 = 4;  // columns a warp sums at once (their loads in flight together)
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    for (int i = tid; i < rows; i += NT) xs[i] = x[i];
    __syncthreads();
    // w_i = x_i + sum_{q>i} V[q][i] x_q
    for (int i0 = w * C4; i0 < k; i0 += NW * C4) {
        T s[C4];
#pragma unroll
        for (int u = 0; u < C4; u++) s[u] = T(0);
        for (int q = i0 + 1 + lane; q < rows; q += 32) {
            const T xq = xs[q];
#pragma unroll
            for (int u = 0; u < C4; u++)
                if (i0 + u < k && q > i0 + u) s[u] += V[q + (size_t)(i0 + u) * ld] * xq;
        }
#pragma unroll
        for (int u = 0; u < C4; u++) {
            const T v = warp_sum(s[u]);
            if (lane == 0 && i0 + u < k) wv[i0 + u] = xs[i0 + u] + v;
        }
    }
    __syncthreads();
    if (trans) {
        // y_i = sum_{j<=i} T[j][i] w_j, lanes down column i of T
        for (int i0 = w * C4; i0 < k; i0 += NW * C4) {
            T s[C4];
#pragma unroll
            for (int u = 0; u < C4; u++) s[u] = T(0);
            const int hi = min(i0 + C4 - 1, k - 1);
            for (int j = lane; j <= hi; j += 32) {
                const T wj = wv[j];
#pragma unroll
                for (int u = 0; u < C4; u++)
                    if (j <= i0 + u && i0 + u < k) s[u] += Tm[j + (size_t)(i0 + u) * ld] * wj;
            }
#pragma unroll
            for (int u = 0; u < C4; u++) {
                const T v = warp_sum(s[u]);
                if (lane == 0 && i0 + u < k) yv[i0 + u] = v;
            }
        }
    } else {
        // y_i = sum_{j>=i} T[i][j] w_j, consecutive threads on consecutive rows of T
        for (int i = tid; i < k; i += NT) {
            T s[8];
#pragma unroll
            for (int u = 0; u < 8; u++) s[u] = T(0);
            int j = i;
            for (; j + 7 < k; j += 8) {
#pragma unroll
                for (int u = 0; u < 8; u++) s[u] += Tm[i + (size_t)(j + u) * ld] * wv[j + u];
            }
            for (; j < k; j++) s[0] += Tm[i + (size_t)j * ld] * wv[j];
            yv[i] = ((s[0] + s[1]) + (s[2] + s[3])) + ((s[4] + s[5]) + (s[6] + s[7]));
        }
    }
    __syncthreads();
    // x_q -= sum_{i <= min(q, k-1)} V[q][i] y_i (V[q][q] = 1), a thread per row
    for (int q = tid; q < rows; q += NT) {
        const int iend = min(q, k);
        T s[8];
#pragma unroll
        for (int u = 0; u < 8; u++) s[u] = T(0);
        int i = 0;
        for (; i + 7 < iend; i += 8) {
#pragma unroll
            for (int u = 0; u < 8; u++) s[u] += V[q + (size_t)(i + u) * ld] * yv[i + u];
        }
        for (; i < iend; i++) s[0] += V[q + (size_t)i * ld] * yv[i];
        if (q < k) s[0] += yv[q];
        x[q] = xs[q] - (((s[0] + s[1]) + (s[2] + s[3])) + ((s[4] + s[5]) + (s[6] + s[7])));
    }
}

// The same Orthogonal op for the large clusters of the top levels, on a thread-block
// cluster of CS CTAs per (cluster, right-hand side): one CTA reads a fraction of V and T
// only, so the op is spread over CS SMs' load bandwidth (one CTA alone is bound by the
// loads it can keep in flight).  CTA r computes w and y for its slice of the k reflectors
// and the update of its slice of the rows; the slices of w and of y are gathered through
// distributed shared memory after a cluster barrier each.  Rows x reflectors of the
// update are split over the warps (row blocks of 32 lanes x reflector chunks, partial
// sums added in chunk order).  Shared memory: x, w, y and the partial sums.
template <typename T, int NT>
__global__ void __launch_bounds__(NT) ortho_cluster_kernel(Ctx<T> c, XCtx<T> X, const DOrtho* __restrict__ items,
                                                           int count, const T* __restrict__ vstore,
                                                           const T* __restrict__ tstore, int trans) {
    pdl_wait_and_release();
    namespace cgx = cooperative_groups;
    cgx::cluster_group cl = cgx::this_cluster();
    const int CS = (int)cl.num_blocks(), me = (int)cl.block_rank();
    const int pair = blockIdx.x / CS;
    const int item = pair % count, r = pair / count;
    const DOrtho it = items[item];
    const int rows = c.rows0[it.cluster];
    const int k = c.csize[it.cluster];
    if (k >= rows || k == 0) return;  // the same for every CTA of the cluster
    const int ld = c.cap[it.cluster];
    const T* __restrict__ V = vstore + it.v_off;
    const T* __restrict__ Tm = tstore + it.v_off;
    T* x = X.xs + X.xoff[it.cluster] + (size_t)r * X.xld;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* xs = reinterpret_cast<T*>(smem_raw);
    T* wv = xs + rows;
    T* yv = wv + k;
    T* part = yv + k;  // NW x 32 partial sums
    constexpr int NW = NT / 32;
    constexpr int C4 = 4;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    auto lo = [&](int n, int q) { return (int)((long long)n * q / CS); };
    // part holds 32 x max(NW, row blocks of a slice) partial sums
    const int i_lo = lo(k, me), i_hi = lo(k, me + 1);
    for (int i = tid; i < rows; i += NT) xs[i] = x[i];
    __syncthreads();
    for (int i0 = i_lo + w * C4; i0 < i_hi; i0 += NW * C4) {
        T s4[C4];
#pragma unroll
        for (int u = 0; u < C4; u++) s4[u] = T(0);
        for (int q = i0 + 1 + lane; q < rows; q += 32) {
            const T xq = xs[q];
#pragma unroll
            for (int u = 0; u < C4; u++)
                if (i0 + u < i_hi && q > i0 + u) s4[u] += V[q + (size_t)(i0 + u) * ld] * xq;
        }
#pragma unroll
        for (int u = 0; u < C4; u++) {
            const T v = warp_sum(s4[u]);
            if (lane == 0 && i0 + u < i_hi) wv[i0 + u] = xs[i0 + u] + v;
        }
    }
    // every reflector's w from the CTA that owns it
    auto owner = [&](int i) {
        int q = (int)(((long long)i * CS) / k);
        while (q + 1 < CS && lo(k, q + 1) <= i) q++;
        while (q > 0 && lo(k, q) > i) q--;
        return q;
    };
    cl.sync();
    for (int i = tid; i < k; i += NT) {
        const int o = owner(i);
        if (o != me) wv[i] = *cl.map_shared_rank(wv + i, o);
    }
    __syncthreads();
    if (trans) {
        for (int i0 = i_lo + w * C4; i0 < i_hi; i0 += NW * C4) {
            T s4[C4];
#pragma unroll
            for (int u = 0; u < C4; u++) s4[u] = T(0);
            const int hi = min(i0 + C4 - 1, i_hi - 1);
            for (int j = lane; j <= hi; j += 32) {
                const T wj = wv[j];
#pragma unroll
                for (int u = 0; u < C4; u++)
                    if (j <= i0 + u && i0 + u < i_hi) s4[u] += Tm[j + (size_t)(i0 + u) * ld] * wj;
            }
#pragma unroll
            for (int u = 0; u < C4; u++) {
                const T v = warp_sum(s4[u]);
                if (lane == 0 && i0 + u < i_hi) yv[i0 + u] = v;
            }
        }
    } else {
        for (int i = i_lo + tid; i < i_hi; i += NT) {
            T s8[8];
#pragma unroll
            for (int u = 0; u < 8; u++) s8[u] = T(0);
            int j = i;
            for (; j + 7 < k; j += 8) {
#pragma unroll
                for (int u = 0; u < 8; u++) s8[u] += Tm[i + (size_t)(j + u) * ld] * wv[j + u];
            }
            for (; j < k; j++) s8[0] += Tm[i + (size_t)j * ld] * wv[j];
            yv[i] = ((s8[0] + s8[1]) + (s8[2] + s8[3])) + ((s8[4] + s8[5]) + (s8[6] + s8[7]));
        }
    }
    cl.sync();
    for (int i = tid; i < k; i += NT) {
        const int o = owner(i);
        if (o != me) yv[i] = *cl.map_shared_rank(yv + i, o);
    }
    __syncthreads();
    // x_q -= sum_{i <= min(q, k-1)} V[q][i] y_i for this CTA's rows: warp w takes row block
    // w mod nrb (32 rows, a lane each) and reflector chunk w / nrb
    const int q_lo = lo(rows, me), q_hi = lo(rows, me + 1);
    const int nrb = (q_hi - q_lo + 31) / 32;
    if (nrb > 0) {
        const int nchunk = max(1, NW / nrb);
        for (int vw = w; vw < nrb * nchunk; vw += NW) {  // more row blocks than warps: in turns
            const int rb = vw % nrb, ch = vw / nrb;
            const int q = q_lo + 32 * rb + lane;
            const int iend = q < q_hi ? min(q, k) : 0;
            const int c0 = (int)((long long)k * ch / nchunk), c1 = (int)((long long)k * (ch + 1) / nchunk);
            const int e = min(c1, iend);
            T s8[8];
#pragma unroll
            for (int u = 0; u < 8; u++) s8[u] = T(0);
            int i = c0;
            for (; i + 7 < e; i += 8) {
#pragma unroll
                for (int u = 0; u < 8; u++) s8[u] += V[q + (size_t)(i + u) * ld] * yv[i + u];
            }
            for (; i < e; i++) s8[0] += V[q + (size_t)i * ld] * yv[i];
            if (q < k && q >= c0 && q < c1) s8[0] += yv[q];  // V[q][q] = 1
            part[ch * (32 * nrb) + 32 * rb + lane] =
                ((s8[0] + s8[1]) + (s8[2] + s8[3])) + ((s8[4] + s8[5]) + (s8[6] + s8[7]));
        }
        __syncthreads();
        for (int qq = tid; qq < q_hi - q_lo; qq += NT) {
            T sum = T(0);
            for (int ch2 = 0; ch2 < nchunk; ch2++) sum += part[ch2 * (32 * nrb) + qq];
            x[q_lo + qq] = xs[q_lo + qq] - sum;
        }
    }
    // no CTA leaves while another may still read its w or y
    cl.sync();
}

// Merge op: parent x = children heads concatenated (fwd) and back (bwd)
template <typename T>
__global__ void merge_x_kernel(Ctx<T> c, XCtx<T> X, const int* __restrict__ children, const int* __restrict__ parent_of,
                               int nchildren, const int* __restrict__ cpos, int fwd) {
    pdl_wait_and_release();
    // a warp per (child, right-hand side)
    const int pair = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (pair >= nchildren * X.nrhs) return;
    const int k = pair % nchildren;
    const int r = pair / nchildren;
    const int ch = children[k];
    const int p = parent_of[k];
    const int n = c.csize[ch];
    T* xc = X.xs + X.xoff[ch] + r * X.xld;
    T* xp = X.xs + X.xoff[p] + cpos[ch] + r * X.xld;
    for (int i = threadIdx.x & 31; i < n; i += 32) {
        if (fwd) xp[i] = xc[i];
        else xc[i] = xp[i];
    }
}

// ------------------------------------------------------------------------------------
// Solve sweeps for many right-hand sides (16 or more).  Right-hand sides in blocks of 32,
// one per lane; factor tiles and x tiles staged in shared memory with coalesced loads, so
// that every factor element is read once per 32 right-hand sides.  8 warps; warp w owns
// the tile rows w + 8u.  Same operations, same order of ops, as the one-right-hand-side
// kernels above; sums within an op run in chunks of MR_KC.
// ------------------------------------------------------------------------------------
constexpr int MR_RB = 32;      // right-hand sides per block (lanes)
constexpr int MR_KC = 32;      // reduction chunk
constexpr int MR_MAXROWS = 64; // rows of one tile (2 * TV_ROWS for single-tile clusters)
constexpr int MR_U = MR_MAXROWS / 8;

// acc[u] += sum_{k in [k0, k1)} F(r0 + w + 8u, k) * x[k][rb0 + lane] with F(i, k) at
// A[i + k*ld] (row_fast) or A[k + i*ld]; pred: 0 all, 1 k < i only, 2 k > i only.
// x column j of the block at xcol + j * xld.  Leaves the tiles free (ends with a barrier).
template <typename T>
__device__ __forceinline__ void mr_accum(T (&acc)[MR_U], const T* __restrict__ A, int ld, bool row_fast, int r0,
                                         int nr, int k0, int k1, int pred, const T* __restrict__ xcol, long long xld,
                                         int nrb, T (*xs)[MR_RB + 1], T (*fs)[MR_KC + 1]) {
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    for (int kb = k0; kb < k1; kb += MR_KC) {
        const int kw = min(MR_KC, k1 - kb);
        for (int idx = tid; idx < MR_KC * MR_RB; idx += blockDim.x) {
            const int kk = idx % MR_KC, j = idx / MR_KC;
            xs[kk][j] = (kk < kw && j < nrb) ? xcol[(kb + kk) + (size_t)j * xld] : T(0);
        }
        if (row_fast) {
            for (int idx = tid; idx < MR_KC * nr; idx += blockDim.x) {
                const int i = idx % nr, kk = idx / nr;
                const int k = kb + kk, row = r0 + i;
                const bool ok = kk < kw && (pred == 0 || (pred == 1 ? k < row : k > row));
                fs[i][kk] = ok ? A[row + (size_t)k * ld] : T(0);
            }
        } else {
            for (int idx = tid; idx < MR_KC * nr; idx += blockDim.x) {
                const int kk = idx % MR_KC, i = idx / MR_KC;
                const int k = kb + kk, row = r0 + i;
                const bool ok = kk < kw && (pred == 0 || (pred == 1 ? k < row : k > row));
                fs[i][kk] = ok ? A[k + (size_t)row * ld] : T(0);
            }
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < MR_KC; kk++) {
            const T xv = xs[kk][lane];
#pragma unroll
            for (int u = 0; u < MR_U; u++)
                if (w + 8 * u < nr) acc[u] += fs[w + 8 * u][kk] * xv;
        }
        __syncthreads();
    }
}

// Triangular products (as trsv4_kernel) for many right-hand sides: one CTA per (cluster,
// row tile), every right-hand-side block in turn; multi-tile clusters go through the
// scratch copy and the last tile copies back.
template <typename T>
__global__ void __launch_bounds__(256) trsv_mrhs_kernel(Ctx<T> c, XCtx<T> X, const int* __restrict__ clusters,
                                                        const int* __restrict__ lblocks,
                                                        const int2* __restrict__ tiles, int trans, T* tmp,
                                                        int* counters) {
    __shared__ T xs[MR_KC][MR_RB + 1];
    __shared__ T fs[MR_MAXROWS][MR_KC + 1];
    const int2 tl = tiles[blockIdx.x];
    const int cl = clusters[tl.x];
    const int n = c.rows0[cl];
    const int nt = n <= 2 * TV_ROWS ? 1 : (n + TV_ROWS - 1) / TV_ROWS;
    if (n == 0 || tl.y >= nt) return;
    const int r0 = nt == 1 ? 0 : tl.y * TV_ROWS, r1 = nt == 1 ? n : min(n, r0 + TV_ROWS), nr = r1 - r0;
    const T* L = bptr(c, lblocks[tl.x]);
    const int ld = c.blk[lblocks[tl.x]].ld;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int rb0 = 0; rb0 < X.nrhs; rb0 += MR_RB) {
        const int nrb = min(MR_RB, X.nrhs - rb0);
        const T* xcol = X.xs + X.xoff[cl] + (size_t)rb0 * X.xld;
        T acc[MR_U];
#pragma unroll
        for (int u = 0; u < MR_U; u++) acc[u] = T(0);
        // forward: L^{-1}[i][k] (k < i) at L[k + i*ld]; backward: L^{-1}[k][i] (k > i) at L[i + k*ld]
        if (!trans) mr_accum(acc, L, ld, false, r0, nr, 0, r1, 1, xcol, X.xld, nrb, xs, fs);
        else mr_accum(acc, L, ld, true, r0, nr, r0 + 1, n, 2, xcol, X.xld, nrb, xs, fs);
        T* ycol = (nt == 1 ? X.xs : tmp) + X.xoff[cl] + (size_t)rb0 * X.xld;
        // through the (free) factor tile, so that consecutive threads write consecutive rows
#pragma unroll
        for (int u = 0; u < MR_U; u++)
            if (w + 8 * u < nr) fs[w + 8 * u][lane] = acc[u];
        __syncthreads();
        for (int idx = threadIdx.x; idx < nr * nrb; idx += blockDim.x) {
            const int i = idx % nr, j = idx / nr, row = r0 + i;
            const size_t o = row + (size_t)j * X.xld;
            ycol[o] = fs[i][j] + xcol[o] / L[row + (size_t)row * ld];
        }
        __syncthreads();
    }
    if (nt == 1) return;
    __threadfence();
    __syncthreads();
    __shared__ int last;
    if (threadIdx.x == 0) last = atomicAdd(&counters[cl], 1) == nt - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    for (int rhs = 0; rhs < X.nrhs; rhs++) {
        const size_t off = X.xoff[cl] + (size_t)rhs * X.xld;
        for (int k = threadIdx.x; k < n; k += blockDim.x) X.xs[off + k] = __ldcg(tmp + off + k);
    }
    if (threadIdx.x == 0) counters[cl] = 0;
}

// Triangular products for many right-hand sides on clusters of at most MR_MAXROWS rows:
// one WARP per (cluster, block of 32 right-hand sides), eight per CTA, no CTA barrier.
// The warp stages its x tile (rows x 32) in shared memory with row-contiguous loads, each
// lane forms its right-hand side's products with broadcast loads of L^{-1} (in place, rows
// in the order that leaves every needed original entry unread-over), and the tile goes back
// with row-contiguous stores.  The thousands of 10-60-row clusters of the lower levels
// were CTA-latency-bound in trsv_mrhs_kernel.
constexpr int MRS_WARPS = 8;

template <typename T>
__global__ void __launch_bounds__(32 * MRS_WARPS) trsv_mrhs_small_kernel(Ctx<T> c, XCtx<T> X,
                                                                        const int* __restrict__ clusters,
                                                                        const int* __restrict__ lblocks,
                                                                        const int* __restrict__ idx, int count,
                                                                        int trans) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    T (*xs)[MR_RB + 1] = reinterpret_cast<T (*)[MR_RB + 1]>(smem_raw) + (size_t)w * MR_MAXROWS;
    const int nrbk = (X.nrhs + MR_RB - 1) / MR_RB;
    const int pair = blockIdx.x * MRS_WARPS + w;
    if (pair >= count * nrbk) return;
    const int k = idx[pair / nrbk], rb0 = (pair % nrbk) * MR_RB;
    const int cl = clusters[k];
    const int n = c.rows0[cl];
    if (n == 0) return;
    const int nrb = min(MR_RB, X.nrhs - rb0);
    const T* L = bptr(c, lblocks[k]);
    const int ld = c.blk[lblocks[k]].ld;
    T* xcol = X.xs + X.xoff[cl] + (size_t)rb0 * X.xld;
    for (int j = 0; j < nrb; j++)
        for (int i = lane; i < n; i += 32) xs[i][j] = xcol[i + (size_t)j * X.xld];
    __syncwarp();
    // The factor entries of a row come in 32-element chunks, one per lane (coalesced when the
    // row is contiguous), and reach every lane by shuffle; every lane runs the loops (lanes
    // past the last right-hand side work on padding and are not written back).
    if (!trans) {
        // y_i = x_i / L_ii + sum_{k<i} L^{-1}[i][k] x_k, L^{-1}[i][k] at L[k + i ld]; rows from
        // the last, so every x_k (k < i) is still the original
        for (int i = n - 1; i >= 0; i--) {
            const T* li = L + (size_t)i * ld;
            T s0 = xs[i][lane] / li[i], s1 = 0;
            for (int q0 = 0; q0 < i; q0 += 32) {
                const T lv = q0 + lane < i ? li[q0 + lane] : T(0);
                const int cnt = min(32, i - q0);
                int u = 0;
                for (; u + 1 < cnt; u += 2) {
                    s0 += __shfl_sync(0xffffffffu, lv, u) * xs[q0 + u][lane];
                    s1 += __shfl_sync(0xffffffffu, lv, u + 1) * xs[q0 + u + 1][lane];
                }
                if (u < cnt) s0 += __shfl_sync(0xffffffffu, lv, u) * xs[q0 + u][lane];
            }
            __syncwarp();
            xs[i][lane] = s0 + s1;
        }
    } else {
        // y_i = x_i / L_ii + sum_{k>i} L^{-1}[k][i] x_k, L^{-1}[k][i] at L[i + k ld]; rows from
        // the first
        for (int i = 0; i < n; i++) {
            T s0 = xs[i][lane] / L[i + (size_t)i * ld], s1 = 0;
            for (int q0 = i + 1; q0 < n; q0 += 32) {
                const T lv = q0 + lane < n ? L[i + (size_t)(q0 + lane) * ld] : T(0);
                const int cnt = min(32, n - q0);
                int u = 0;
                for (; u + 1 < cnt; u += 2) {
                    s0 += __shfl_sync(0xffffffffu, lv, u) * xs[q0 + u][lane];
                    s1 += __shfl_sync(0xffffffffu, lv, u + 1) * xs[q0 + u + 1][lane];
                }
                if (u < cnt) s0 += __shfl_sync(0xffffffffu, lv, u) * xs[q0 + u][lane];
            }
            __syncwarp();
            xs[i][lane] = s0 + s1;
        }
    }
    __syncwarp();
    for (int j = 0; j < nrb; j++)
        for (int i = lane; i < n; i += 32) xcol[i + (size_t)j * X.xld] = xs[i][j];
}

// Gemm sweeps (as gemm_fwd2 / gemm_bwd2) for many right-hand sides: one CTA per (group,
// 32 rows of the updated slot), ops of the group in order, all right-hand-side blocks.
// fwd: x_n -= A_ns x_s (kind 1, A[i + j*ld]) or A_sn^T x_s (kind 2, A[j + i*ld]);
// bwd: x_s -= A_ns^T x_n (kind 1, A[j + i*ld]) or A_sn x_n (kind 2, A[i + j*ld]).
template <typename T>
__global__ void __launch_bounds__(256) gemm_mrhs_kernel(Ctx<T> c, XCtx<T> X, const DGroup* __restrict__ groups,
                                                        const DGemmOp* __restrict__ ops,
                                                        const DTile* __restrict__ tiles, int fwd) {
    __shared__ T xs[MR_KC][MR_RB + 1];
    __shared__ T fs[MR_MAXROWS][MR_KC + 1];
    const DTile tl = tiles[blockIdx.x];
    const DGroup G = groups[tl.item];
    const int key = G.key;
    const int nk = fwd ? c.rows0[key] : c.csize[key];
    const int i0 = tl.tile_i * 32;
    if (i0 >= nk) return;
    const int nr = min(32, nk - i0);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    T* ycol0 = X.xs + X.xoff[key];
    for (int rb0 = 0; rb0 < X.nrhs; rb0 += MR_RB) {
        const int nrb = min(MR_RB, X.nrhs - rb0);
        T acc[MR_U];
#pragma unroll
        for (int u = 0; u < MR_U; u++) acc[u] = T(0);
        for (int o = 0; o < G.count; o++) {
            const DGemmOp op = ops[G.first + o];
            const int other = fwd ? op.self : op.nbr;
            const int nj = fwd ? c.csize[op.self] : c.rows0[op.nbr];
            const T* xcol = X.xs + X.xoff[other] + (size_t)rb0 * X.xld;
            const bool row_fast = fwd ? op.kind == 1 : op.kind == 2;
            mr_accum(acc, bptr(c, op.block), c.blk[op.block].ld, row_fast, i0, nr, 0, nj, 0, xcol, X.xld, nrb, xs,
                     fs);
        }
        // through the (free) factor tile, so that consecutive threads update consecutive rows
#pragma unroll
        for (int u = 0; u < MR_U; u++)
            if (w + 8 * u < nr) fs[w + 8 * u][lane] = acc[u];
        __syncthreads();
        for (int idx = threadIdx.x; idx < nr * nrb; idx += blockDim.x) {
            const int i = idx % nr, j = idx / nr;
            ycol0[(i0 + i) + (size_t)(rb0 + j) * X.xld] -= fs[i][j];
        }
        __syncthreads();
    }
}

// Orthogonal op (as ortho_wyb_kernel) for many right-hand sides: one CTA per cluster, x of
// a right-hand-side block resident in shared memory (rows x 33), every 32-reflector block:
// W = V_b^T X, Y = T_b^T W or T_b W, X -= V_b Y.
template <typename T>
__global__ void __launch_bounds__(256) ortho_mrhs_kernel(Ctx<T> c, XCtx<T> X, const DOrtho* __restrict__ items,
                                                         const T* vstore, const T* tstore, int trans) {
    __shared__ T vt[MR_KC][QB + 1];
    __shared__ T Wm[QB][MR_RB + 1];
    __shared__ T Ym[QB][MR_RB + 1];
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T (*Xs)[MR_RB + 1] = reinterpret_cast<T (*)[MR_RB + 1]>(smem_raw);
    const DOrtho it = items[blockIdx.x];
    const int rows = c.rows0[it.cluster];
    const int k = c.csize[it.cluster];
    if (k >= rows || k == 0) return;
    const int ld = c.cap[it.cluster];
    const T* V = vstore + it.v_off;
    const T* Tm = tstore + it.v_off;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int nb = (k + QB - 1) / QB;
    for (int rb0 = 0; rb0 < X.nrhs; rb0 += MR_RB) {
        const int nrb = min(MR_RB, X.nrhs - rb0);
        T* xcol = X.xs + X.xoff[it.cluster] + (size_t)rb0 * X.xld;
        __syncthreads();
        for (int idx = tid; idx < rows * MR_RB; idx += blockDim.x) {
            const int r = idx % rows, j = idx / rows;
            Xs[r][j] = j < nrb ? xcol[r + (size_t)j * X.xld] : T(0);
        }
        for (int q = 0; q < nb; q++) {
            const int b = trans ? q : nb - 1 - q;
            const int i0 = b * QB, bw = min(QB, k - i0);
            // W[i][l] = sum_{r >= i0+i} v_i[r] X[r][l]   (v_i[i0+i] = 1)
            T acc[4] = {0, 0, 0, 0};
            for (int rb = i0; rb < rows; rb += MR_KC) {
                __syncthreads();
                for (int idx = tid; idx < MR_KC * QB; idx += blockDim.x) {
                    const int kk = idx % MR_KC, ii = idx / MR_KC;
                    const int r = rb + kk, col = i0 + ii;
                    T v = T(0);
                    if (ii < bw && r < rows) v = r > col ? V[r + (size_t)col * ld] : (r == col ? T(1) : T(0));
                    vt[kk][ii] = v;
                }
                __syncthreads();
                const int kw = min(MR_KC, rows - rb);
                for (int kk = 0; kk < kw; kk++) {
                    const T xv = Xs[rb + kk][lane];
#pragma unroll
                    for (int u = 0; u < 4; u++) acc[u] += vt[kk][w + 8 * u] * xv;
                }
            }
#pragma unroll
            for (int u = 0; u < 4; u++) Wm[w + 8 * u][lane] = acc[u];
            __syncthreads();
            // Y = T_b^T W (fwd) or T_b W (bwd)
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int i = w + 8 * u;
                T y = T(0);
                if (i < bw) {
                    if (trans)
                        for (int j = 0; j <= i; j++) y += Tm[(i0 + j) + (size_t)(i0 + i) * ld] * Wm[j][lane];
                    else
                        for (int j = i; j < bw; j++) y += Tm[(i0 + i) + (size_t)(i0 + j) * ld] * Wm[j][lane];
                }
                Ym[i][lane] = y;
            }
            __syncthreads();
            // X[r][l] -= sum_i v_i[r] Y[i][l]
            for (int rb = i0; rb < rows; rb += MR_KC) {
                __syncthreads();
                for (int idx = tid; idx < MR_KC * QB; idx += blockDim.x) {
                    const int kk = idx % MR_KC, ii = idx / MR_KC;
                    const int r = rb + kk, col = i0 + ii;
                    T v = T(0);
                    if (ii < bw && r < rows) v = r > col ? V[r + (size_t)col * ld] : (r == col ? T(1) : T(0));
                    vt[kk][ii] = v;
                }
                __syncthreads();
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const int kk = w + 8 * u;
                    if (rb + kk < rows) {
                        T s2 = T(0);
                        for (int ii = 0; ii < QB; ii++) s2 += vt[kk][ii] * Ym[ii][lane];
                        Xs[rb + kk][lane] -= s2;
                    }
                }
            }
        }
        __syncthreads();
        for (int idx = tid; idx < rows * MR_RB; idx += blockDim.x) {
            const int r = idx % rows, j = idx / rows;
            if (j < nrb) xcol[r + (size_t)j * X.xld] = Xs[r][j];
        }
    }
}

// Merge op for many right-hand sides: one CTA per child, every right-hand side.
template <typename T>
__global__ void merge_x_mrhs_kernel(Ctx<T> c, XCtx<T> X, const int* __restrict__ children,
                                    const int* __restrict__ parent_of, const int* __restrict__ cpos, int fwd) {
    const int ch = children[blockIdx.x];
    const int p = parent_of[blockIdx.x];
    const int n = c.csize[ch];
    for (int idx = threadIdx.x; idx < n * X.nrhs; idx += blockDim.x) {
        const int i = idx % n, r = idx / n;
        T* xc = X.xs + X.xoff[ch] + (size_t)r * X.xld;
        T* xp = X.xs + X.xoff[p] + cpos[ch] + (size_t)r * X.xld;
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

// y += a x
__global__ void axpy_kernel(int n, double a, const double* __restrict__ x, double* __restrict__ y) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) y[i] += a * x[i];
}

__global__ void sub_kernel(int n, const double* a, const double* b, double* y) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) y[i] = a[i] - b[i];
}

// Several right-hand sides at once: column j of every n x k operand at offset j * n
// (blockIdx.y = j), the same per-column arithmetic and reduction order as the kernels above.
// Scalars of column j at sc[8 * j + slot] (slots as above, [4] b.b); active[j] == 0 freezes
// a converged column.
__global__ void spmv_multi_kernel(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                                  const double* __restrict__ v, const double* __restrict__ x, double* __restrict__ y) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n) return;
    const size_t off = (size_t)blockIdx.y * n;
    double s = 0;
    for (int k = rp[row]; k < rp[row + 1]; k++) s += v[k] * x[off + ci[k]];
    y[off + row] = s;
}

__global__ void dot_multi_partial_kernel(int n, const double* __restrict__ a, const double* __restrict__ b,
                                         double* partial) {
    __shared__ double red[33];
    const size_t off = (size_t)blockIdx.y * n;
    double s = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        s += a[off + i] * b[off + i];
    s = block_sum(s, red);
    if (threadIdx.x == 0) partial[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = s;
}

__global__ void dot_multi_final_kernel(const double* partial, int np, double* sc, int slot) {
    __shared__ double red[33];
    double s = 0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) s += partial[(size_t)blockIdx.x * np + i];
    s = block_sum(s, red);
    if (threadIdx.x == 0) sc[8 * blockIdx.x + slot] = s;
}

__global__ void cg_multi_update_xr_kernel(int n, double* x, double* r, const double* p, const double* Ap,
                                          const double* sc, const int* active) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (i >= n || !active[j]) return;
    const size_t o = (size_t)j * n + i;
    const double alpha = sc[8 * j] / sc[8 * j + 1];
    x[o] += alpha * p[o];
    r[o] -= alpha * Ap[o];
}

__global__ void cg_multi_update_p_kernel(int n, double* p, const double* z, const double* sc, const int* active) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (i >= n || !active[j]) return;
    const size_t o = (size_t)j * n + i;
    const double beta = sc[8 * j] / sc[8 * j + 3];
    p[o] = z[o] + beta * p[o];
}

__global__ void copy_scalar_multi_kernel(double* sc, int k, int dst, int src) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < k) sc[8 * j + dst] = sc[8 * j + src];
}

__global__ void sub_multi_kernel(int n, const double* a, const double* b, double* y) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t o = (size_t)blockIdx.y * n + i;
    y[o] = a[o] - b[o];
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
// Allocation-free solve: fixed scratch for the per-cluster solve vectors
// ------------------------------------------------------------------------------------
// Some callers cannot allocate device memory at the moment they need a solve: code that
// is being captured into a CUDA graph (cudaMalloc is not allowed while a stream captures
// in the global or thread-local mode), code running under a fixed memory budget that
// preallocates everything up front, or a host framework that owns the device allocator.
// For them the solve can use this array instead of vectors owned by the factor.  It is
// part of the library image, so every GPU that loads the library holds these 16 MiB
// until the process exits.  All calls share it: two allocation-free solves that overlap
// on the GPU (different streams, or different trees on different streams) race on it.
// Nothing in it has to start at zero: every slot a solve reads was written earlier in the
// same solve.
constexpr size_t kNoAllocSolveScratchBytes = size_t(16) << 20;
static __device__ __align__(256) unsigned char g_noalloc_solve_scratch[kNoAllocSolveScratchBytes];

constexpr int kMaxDevices = 64;
static void* g_noalloc_scratch_addr[kMaxDevices];
static std::once_flag g_noalloc_scratch_once[kMaxDevices];

// Device address of the scratch array on device `dev`.  In host code the array's name is
// only a host-side stand-in, so the address is looked up with cudaGetSymbolAddress, once
// per device, with that device current (the first allocation-free solve on a device does
// this; make that first call before any stream capture).  The caller has made `dev` (the
// tree's device) current; a different current device is refused rather than resolved.
static void* noalloc_solve_scratch(int dev) {
    if (dev < 0 || dev >= kMaxDevices) throw DeviceError{SPAND_ERR_UNSUPPORTED, "device index out of range"};
    if (current_device() != dev)
        throw DeviceError{SPAND_ERR_STATE, "allocation-free solve: the tree's device is not the current device"};
    std::call_once(g_noalloc_scratch_once[dev], [dev] {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_solve_scratch);
        if (e != cudaSuccess || p == nullptr)
            throw DeviceError{SPAND_ERR_CUDA, std::string("cudaGetSymbolAddress(solve scratch): ") + cudaGetErrorString(e)};
        g_noalloc_scratch_addr[dev] = p;
    });
    return g_noalloc_scratch_addr[dev];
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
    // the current device is the tree's: every later call runs with it current
    DeviceFactor(cudaStream_t s, const std::vector<int>& perm) : s_(s), perm_h_(perm), dev_(current_device()) {}
    ~DeviceFactor() override {
        drop_factor_graph();
        for (cudaEvent_t e : tune_ev_) cudaEventDestroy(e);
        if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
        if (graph_) cudaGraphDestroy(graph_);
        if (xs_) cudaFree(xs_);
        if (h_status_) cudaFreeHost(h_status_);
        if (ev_fork_) cudaEventDestroy(ev_fork_);
        if (ev_join_) cudaEventDestroy(ev_join_);
        if (s2_) cudaStreamDestroy(s2_);
        for (void* p : owned_) cudaFree(p);
    }

    int precision_bytes() const override { return sizeof(T); }
    cudaStream_t stream() const override { return s_; }
    size_t device_bytes() const override { return bytes_; }

    void upload(const Plan& P, const std::vector<int64_t>& amap) override {
        P_ = &P;
        nc_ = P.nclusters;
        lu_ = P.lu;
        ldlt_ = P.ldlt;
        lorasp_ = P.lorasp;
        if (lorasp_) {
            std::vector<int4> sp;
            for (const LoraSplit& s : P.lr_splits) sp.push_back(make_int4(s.block, s.nbr, s.transposed, s.sblock));
            lr_splits_ = up(sp);
        }
        init_qrcp_limits();
        SPAND_CUDA(cudaStreamCreateWithFlags(&s2_, cudaStreamNonBlocking));
        SPAND_CUDA(cudaEventCreateWithFlags(&ev_fork_, cudaEventDisableTiming));
        SPAND_CUDA(cudaEventCreateWithFlags(&ev_join_, cudaEventDisableTiming));
        arena_ = alloc<T>(P.arena_len);
        pristine_ = alloc<T>(P.assembled_len);
        amap_n_ = (int64_t)amap.size();
        d_amap_ = up(std::vector<long long>(amap.begin(), amap.end()));
        d_vals_ = alloc<double>(std::max<int64_t>(amap_n_, 1));
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
        tstore_ = alloc<T>(std::max<int64_t>(P.v_len, 1));
        taustore_ = alloc<T>(std::max<int64_t>(P.tau_len, 1));
        tauws_ = alloc<T>(std::max<int64_t>(P.tau_len, 1));
        ws_ = alloc<T>(std::max<int64_t>(P.ws_len, 1));
        ws2_ = alloc<T>(std::max<int64_t>(P.ws_len, 1));
        ws_len_ = std::max<int64_t>(P.ws_len, 1);
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
            // LLT pivots of at most 32 rows: a warp each (potrf_small_kernel)
            // and the others, for the one-CTA kernel when the small ones go to the warp kernel
            auto small_pivots = [&](const std::vector<int>& cl, const std::vector<int>& pv, int*& scl, int*& spv,
                                    int& ns, int*& bcl, int*& bpv, int& nb) {
                std::vector<int> a, b, c2, d2;
                if (!lu_ && !ldlt_)
                    for (size_t q = 0; q < cl.size(); q++) {
                        if (P.c_cap[cl[q]] <= 32) {
                            a.push_back(cl[q]);
                            b.push_back(pv[q]);
                        } else {
                            c2.push_back(cl[q]);
                            d2.push_back(pv[q]);
                        }
                    }
                ns = (int)a.size();
                scl = up(a);
                spv = up(b);
                nb = (int)c2.size();
                bcl = up(c2);
                bpv = up(d2);
            };
            small_pivots(L.elim_clusters, L.elim_pivots, D.elim_ps_cl, D.elim_ps_piv, D.n_elim_ps, D.elim_pb_cl,
                         D.elim_pb_piv, D.n_elim_pb);
            D.elim_smem = smem_for(L.elim_clusters, P);
            D.elim_tri = build_trtri(L.elim_clusters, P);
            // PLU: the panels are products with the inverse block
            build_trsm(L.elim_trsm, lu_ ? L.elim_inv : L.elim_pivots, L.elim_clusters, P, D.elim_trsm0, D.elim_trsm1);
            if (lu_) {
                D.elim_inv = up(L.elim_inv);
                D.elim_lu_smem = lu_smem_for(L.elim_clusters, P);
            }
            if (ldlt_) {
                D.elim_lu_smem = lu_smem_for(L.elim_clusters, P);
                if (D.n_elim && !D.elim_trsm0.smem) throw DeviceError{SPAND_ERR_UNSUPPORTED, "pivot too large for the LDLT panels"};
            }
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
            small_pivots(L.scale_clusters, L.scale_pivots, D.scale_ps_cl, D.scale_ps_piv, D.n_scale_ps, D.scale_pb_cl,
                         D.scale_pb_piv, D.n_scale_pb);
            D.scale_smem = smem_for(L.scale_clusters, P);
            D.scale_tri = build_trtri(L.scale_clusters, P);
            build_trsm(L.scale_trsm, lu_ ? L.scale_inv : L.scale_pivots, L.scale_clusters, P, D.scale_trsm0,
                       D.scale_trsm1);
            if (lu_) {
                D.scale_inv = up(L.scale_inv);
                D.scale_lu_smem = lu_smem_for(L.scale_clusters, P);
            }
            if (lorasp_) D.scale_newpiv = up(L.scale_newpiv);
            if (ldlt_) {
                D.scale_newpiv = up(L.scale_newpiv);
                D.scale_lu_smem = lu_smem_for(L.scale_clusters, P);
                if (D.n_scale && !D.scale_trsm0.smem)
                    throw DeviceError{SPAND_ERR_UNSUPPORTED, "pivot too large for the LDLT panels"};
            }
            {
                std::vector<int> all;
                if (lorasp_) all = L.snap;  // the wave's own clusters
                else
                    for (int cl = 0; cl < nc_; cl++)
                        if (P.c_hlevel[cl] == l) all.push_back(cl);
                D.n_level = (int)all.size();
                D.level_clusters = up(all);
            }
            for (const auto& wave : L.waves) {
                WaveDev W = make_wave(wave);
                max_cols = std::max(max_cols, W.cols);
                max_items = std::max(max_items, W.n);
                if (ldlt_) {
                    // the sign pivot's Q^T D Q split, the sibling's LDL^T, the edge's panel and
                    // the Schur update of the cluster's pivot (tree.cpp:1069-1097, 1340-1341)
                    std::vector<int> sib, sibp, aso, piv;
                    std::vector<DTrsm> tr;
                    std::vector<int> ext;
                    std::vector<DTarget> tg;
                    std::vector<DUpd> uu;
                    std::vector<DTile> tiles;
                    int mx = 1;
                    for (const SparsifyItem& it : wave) {
                        sib.push_back(it.sib);
                        sibp.push_back(it.sib_piv);
                        aso.push_back(it.aso);
                        piv.push_back(it.piv);
                        tr.push_back({it.aso, it.sib_piv, it.sib, 0});
                        ext.push_back(P.c_cap[it.cluster]);
                        const int t = (int)tg.size();
                        tg.push_back({it.piv, 1, (int)uu.size(), 1});
                        uu.push_back({it.aso, 1, it.aso, 0, it.sib});
                        const int nt = (P.c_cap[it.cluster] + ST - 1) / ST;
                        for (int a = 0; a < nt; a++)
                            for (int b = 0; b <= a; b++) tiles.push_back({t, a, b});
                        mx = std::max(mx, P.c_cap[it.cluster]);
                    }
                    W.sib = up(sib);
                    W.sib_piv = up(sibp);
                    W.aso = up(aso);
                    W.piv = up(piv);
                    auto tt = tiles_1d(ext, TRB);
                    W.sib_trsm = {up(tr), up(tt), (int)tt.size(), 0, trsm_smem_n(mx)};
                    if (!W.sib_trsm.smem) throw DeviceError{SPAND_ERR_UNSUPPORTED, "cluster too large for the LDLT panels"};
                    W.sib_targets = up(tg);
                    W.sib_ups = up(uu);
                    W.sib_tiles = up(tiles);
                    W.n_sib_tiles = (int)tiles.size();
                    W.ldlt_smem = lu_smem_n(mx);
                }
                if (lorasp_) {
                    // the siblings and the original edges they take rows from
                    std::vector<int> sib;
                    std::vector<int2> rg;
                    W.stiles = 1;
                    for (const SparsifyItem& it : wave) {
                        sib.push_back(it.sib);
                        rg.push_back(make_int2(it.ofirst, it.ocount));
                        std::vector<int> caps;
                        for (int q = 0; q < it.ocount; q++) caps.push_back(P.c_cap[P.lr_splits[it.ofirst + q].nbr]);
                        W.stiles = std::max(W.stiles, lorasp_split_tiles(caps.data(), it.ocount));
                    }
                    W.sib = up(sib);
                    W.orng = up(rg);
                }
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
                auto tv = [&](const std::vector<int>& cl, int& count) {
                    std::vector<int2> t;
                    for (size_t k = 0; k < cl.size(); k++) {
                        const int cap = P.c_cap[cl[k]];
                        const int nt = cap <= 2 * TV_ROWS ? 1 : (cap + TV_ROWS - 1) / TV_ROWS;
                        for (int q = 0; q < nt; q++) t.push_back(make_int2((int)k, q));
                    }
                    count = (int)t.size();
                    return up(t);
                };
                D.elim_tv = tv(L.op_elim_llt, D.n_elim_tv);
                D.scale_tv = tv(L.op_scale_llt, D.n_scale_tv);
                // many right-hand sides: clusters of at most MR_MAXROWS rows go to the warp
                // kernel, the others keep the row tiles
                auto split = [&](const std::vector<int>& cl, int*& small, int& nsmall, int2*& big, int& nbig) {
                    std::vector<int> s;
                    std::vector<int2> t;
                    for (size_t k = 0; k < cl.size(); k++) {
                        const int cap = P.c_cap[cl[k]];
                        if (cap <= MR_MAXROWS) {
                            s.push_back((int)k);
                            continue;
                        }
                        const int nt = (cap + TV_ROWS - 1) / TV_ROWS;
                        for (int q = 0; q < nt; q++) t.push_back(make_int2((int)k, q));
                    }
                    nsmall = (int)s.size();
                    small = up(s);
                    nbig = (int)t.size();
                    big = up(t);
                };
                split(L.op_elim_llt, D.elim_small, D.n_elim_small, D.elim_big_tv, D.n_elim_big_tv);
                split(L.op_scale_llt, D.scale_small, D.n_scale_small, D.scale_big_tv, D.n_scale_big_tv);
            }
            {
                // Gemm ops grouped: forward by neighbour in op order, backward by
                // eliminated cluster in reverse op order.
                std::map<int, std::vector<DGemmOp>> fwd, bwd;
                std::vector<int> fkeys, bkeys;
                // PLU: GemmOut (6) acts in the forward sweep only, as GemmSymmOut does there;
                // GemmIn (7) in the backward sweep only, as GemmSymmIn does there
                // (operations.cpp:85-110)
                for (const GemmOpItem& g : L.op_gemm) {
                    if (g.kind == 7) continue;
                    if (!fwd.count(g.nbr)) fkeys.push_back(g.nbr);
                    fwd[g.nbr].push_back({g.self, g.nbr, g.block, g.kind == 6 ? 1 : g.kind});
                }
                for (auto it = L.op_gemm.rbegin(); it != L.op_gemm.rend(); ++it) {
                    if (it->kind == 6) continue;
                    if (!bwd.count(it->self)) bkeys.push_back(it->self);
                    bwd[it->self].push_back({it->self, it->nbr, it->block, it->kind == 7 ? 2 : it->kind});
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
                std::vector<int> ef, eb;
                for (const DGroup& g : fg) ef.push_back(P.c_cap[g.key]);
                for (const DGroup& g : bg) eb.push_back(P.c_cap[g.key]);
                auto tf = tiles_1d(ef, GF_ROWS), tb = tiles_1d(eb, GB_ROWS);
                D.gf_tiles = up(tf);
                D.n_gf_tiles = (int)tf.size();
                D.gb_tiles = up(tb);
                D.n_gb_tiles = (int)tb.size();
                auto tf32 = tiles_1d(ef, 32);
                D.gf_tiles32 = up(tf32);
                D.n_gf_tiles32 = (int)tf32.size();
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
                if (ldlt_) {
                    std::vector<int> sibs, owners, spiv;
                    std::map<int, std::vector<DGemmOp>> fwd, bwd;
                    std::vector<int> fk, bk;
                    for (const auto& wave : L.waves)
                        for (const SparsifyItem& it : wave) {
                            sibs.push_back(it.sib);
                            owners.push_back(it.cluster);
                            spiv.push_back(it.sib_piv);
                            // GemmSymmIn(sibling, cluster) with the sibling's signs
                            fk.push_back(it.cluster);
                            fwd[it.cluster].push_back({it.sib, it.cluster, it.aso, 2});
                            bk.push_back(it.sib);
                            bwd[it.sib].push_back({it.sib, it.cluster, it.aso, 2});
                        }
                    D.n_sib = (int)sibs.size();
                    D.sib_clusters = up(sibs);
                    D.sib_owner = up(owners);
                    D.sib_piv = up(spiv);
                    D.x_smem_sib = xsmem_for(sibs, P);
                    {
                        std::vector<int2> t;
                        for (size_t k = 0; k < sibs.size(); k++) {
                            const int cap = P.c_cap[sibs[k]];
                            const int nt = cap <= 2 * TV_ROWS ? 1 : (cap + TV_ROWS - 1) / TV_ROWS;
                            for (int q = 0; q < nt; q++) t.push_back(make_int2((int)k, q));
                        }
                        D.n_sib_tv = (int)t.size();
                        D.sib_tv = up(t);
                    }
                    std::vector<DGroup> fg, bg;
                    std::vector<DGemmOp> fo, bo;
                    std::vector<int> ef, eb;
                    for (int k : fk) {
                        fg.push_back({k, (int)fo.size(), (int)fwd[k].size()});
                        fo.insert(fo.end(), fwd[k].begin(), fwd[k].end());
                        ef.push_back(P.c_cap[k]);
                    }
                    for (int k : bk) {
                        bg.push_back({k, (int)bo.size(), (int)bwd[k].size()});
                        bo.insert(bo.end(), bwd[k].begin(), bwd[k].end());
                        eb.push_back(P.c_cap[k]);
                    }
                    D.sib_gf = up(fg);
                    D.sib_gfo = up(fo);
                    D.sib_gb = up(bg);
                    D.sib_gbo = up(bo);
                    auto tf = tiles_1d(ef, GF_ROWS), tb = tiles_1d(eb, GB_ROWS);
                    D.sib_gf_tiles = up(tf);
                    D.n_sib_gf_tiles = (int)tf.size();
                    D.sib_gb_tiles = up(tb);
                    D.n_sib_gb_tiles = (int)tb.size();
                    for (int c0 : L.op_elim_llt) diag_h_.push_back(c0);
                    for (int c0 : L.op_scale_llt) diag_h_.push_back(c0);
                    for (int c0 : sibs) diag_h_.push_back(c0);
                } else if (lorasp_) {
                    // the siblings' GemmSymmIn ops: forward grouped by neighbour, backward by
                    // sibling, in recording order; kind bit 16: the neighbour's size is its rank
                    std::vector<int> sibs, owners;
                    std::map<int, std::vector<DGemmOp>> fwd, bwd;
                    std::vector<int> fk, bk;
                    for (const auto& wave : L.waves)
                        for (const SparsifyItem& it : wave) {
                            sibs.push_back(it.sib);
                            owners.push_back(it.cluster);
                            for (int q = 0; q < it.scount; q++) {
                                const LoraSibOp& op = P.lr_sibops[it.sfirst + q];
                                const DGemmOp g{it.sib, op.nbr, op.block, 2 | (op.cur ? 16 : 0)};
                                if (!fwd.count(op.nbr)) fk.push_back(op.nbr);
                                fwd[op.nbr].push_back(g);
                                if (!bwd.count(it.sib)) bk.push_back(it.sib);
                                bwd[it.sib].push_back(g);
                            }
                        }
                    D.n_sib = (int)sibs.size();
                    D.sib_clusters = up(sibs);
                    D.sib_owner = up(owners);
                    std::vector<DGroup> fg, bg;
                    std::vector<DGemmOp> fo, bo;
                    std::vector<int> ef, eb;
                    for (int k : fk) {
                        fg.push_back({k, (int)fo.size(), (int)fwd[k].size()});
                        fo.insert(fo.end(), fwd[k].begin(), fwd[k].end());
                        ef.push_back(P.c_cap[k]);
                    }
                    for (int k : bk) {
                        auto& ops = bwd[k];
                        std::reverse(ops.begin(), ops.end());  // backward: reverse recording order
                        bg.push_back({k, (int)bo.size(), (int)ops.size()});
                        bo.insert(bo.end(), ops.begin(), ops.end());
                        eb.push_back(P.c_cap[k]);
                    }
                    D.sib_gf = up(fg);
                    D.sib_gfo = up(fo);
                    D.sib_gb = up(bg);
                    D.sib_gbo = up(bo);
                    auto tf = tiles_1d(ef, GF_ROWS), tb = tiles_1d(eb, GB_ROWS);
                    D.sib_gf_tiles = up(tf);
                    D.n_sib_gf_tiles = (int)tf.size();
                    D.sib_gb_tiles = up(tb);
                    D.n_sib_gb_tiles = (int)tb.size();
                }
                // the x range, and where they fit the staged T_b and V_b tiles
                {
                    const int64_t full = ((int64_t)mx + QB * (QB + 1) + (int64_t)QB * mx) * (int64_t)sizeof(T);
                    D.x_smem_ortho = full <= 200 * 1024 ? (int)full : mx * (int)sizeof(T);
                    // the whole-T form: x, w and y (k <= rows <= capacity)
                    const int64_t of = 3 * (int64_t)mx * (int64_t)sizeof(T);
                    D.ortho_full_smem = of <= 200 * 1024 ? (int)of : 0;
                    D.ortho_full_wide = mx >= 96;
                    // the large clusters of the top levels: CS CTAs per cluster (at least 24
                    // rows each, about eight CTAs per SM in all), 256 threads
                    int cs = 1;
                    while (cs < 8 && mx / (2 * cs) >= 24 && (int64_t)D.n_ortho * cs < 8 * (int64_t)num_sms_) cs *= 2;
                    const int64_t oc = ((int64_t)3 * mx + 32 * std::max<int64_t>(8, (mx / cs + 31) / 32 + 1)) *
                                       (int64_t)sizeof(T);
                    D.ortho_cs = (mx >= 96 && cs > 1 && oc <= 200 * 1024) ? cs : 1;
                    D.ortho_cs_smem = (int)oc;
                }
                const int64_t mr = (int64_t)mx * (MR_RB + 1) * (int64_t)sizeof(T);
                D.ortho_mrhs_smem = mr <= 200 * 1024 ? (int)mr : 0;
            }
        }
        jpvt_ = alloc<int>(max_cols);
        ipvt_ = alloc<int>(max_cols);
        cols_len_ = max_cols;
        if (lu_ || ldlt_) {
            lu_perm_ = alloc<int>(std::max<int64_t>(P.x_len, 1));
            lu_swp_ = alloc<int>(std::max<int64_t>(P.x_len, 1));
        }
        if (ldlt_) {
            signs_ = alloc<T>(std::max<int64_t>(P.x_len, 1));
            diag_ = up(diag_h_);
            n_diag_ = (int)diag_h_.size();
            int mx = 1;
            for (int c0 : diag_h_) mx = std::max(mx, P.c_cap[c0]);
            diag_smem_ = mx * (int)sizeof(T);
        }
        colcount_ = alloc<int>(max_items);
        d_xoff_ = up(std::vector<long long>(P.c_xoff.begin(), P.c_xoff.end()));
        xld_ = P.x_len;
        {
            std::vector<long long> slot(perm_h_.size());
            for (int c0 = 0; c0 < P.nclusters_h; c0++)
                if (P.c_hlevel[c0] == 0)
                    for (int i = 0; i < P.c_cap[c0]; i++) slot[P.c_start[c0] + i] = P.c_xoff[c0] + i;
            d_slot_ = up(slot);
            d_perm_ = up(perm_h_);
        }
        ctx_ = Ctx<T>{arena_, d_blk_, csize_, rows0_, d_cap_, status_};
        SPAND_CUDA(cudaFuncSetAttribute(potrf3_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, POTRF_SMEM_MAX));
        SPAND_CUDA(cudaFuncSetAttribute(trtri_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        SPAND_CUDA(cudaFuncSetAttribute(trsm3_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        if (ldlt_) {
            SPAND_CUDA(cudaFuncSetAttribute(ldlt_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
            SPAND_CUDA(cudaFuncSetAttribute(perm_x_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        }
        if (lu_) {
            SPAND_CUDA(cudaFuncSetAttribute(getrf_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
            SPAND_CUDA(cudaFuncSetAttribute(lu_trsm_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
            SPAND_CUDA(cudaFuncSetAttribute(lu_apply_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        }
        fallback_ = alloc<int>(max_items);
        items_len_ = max_items;
        SPAND_CUDA(cudaFuncSetAttribute(trsv4_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        SPAND_CUDA(cudaFuncSetAttribute(trsv_fused_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        SPAND_CUDA(cudaFuncSetAttribute(ortho_mrhs_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        SPAND_CUDA(cudaFuncSetAttribute(trsv_mrhs_small_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        MRS_WARPS * MR_MAXROWS * (MR_RB + 1) * (int)sizeof(T)));
        tv_count_ = alloc<int>(nc_);
        {
            int mx = 1;
            for (const LevelPlan& L : P.levels)
                mx = std::max(mx, (int)std::max(L.elim_clusters.size(), L.scale_clusters.size()));
            pc_fallback_ = alloc<int>(mx);
        }
        SPAND_CUDA(cudaMemsetAsync(tv_count_, 0, (size_t)std::max(nc_, 1) * sizeof(int), s_));
        SPAND_CUDA(cudaFuncSetAttribute(sparsify_wy_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        larft_smem_elems() * (int)sizeof(T)));
        SPAND_CUDA(cudaFuncSetAttribute(ortho_wyb_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        SPAND_CUDA(cudaFuncSetAttribute(ortho_full_kernel<T, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        200 * 1024));
        SPAND_CUDA(cudaFuncSetAttribute(trsm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        SPAND_CUDA(cudaFuncSetAttribute(ortho_cluster_kernel<T, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        200 * 1024));
        SPAND_CUDA(cudaFuncSetAttribute(ortho_full_kernel<T, 512>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        200 * 1024));
        caps_h_ = P.c_cap;
    }

    void assemble_values(const double* vals, int64_t nnz, bool on_device) override {
        if (nnz != amap_n_) throw DeviceError{SPAND_ERR_ARG, "values do not match the assembled pattern"};
        if (nnz > 0) SPAND_CUDA(cudaMemcpyAsync(d_vals_, vals, nnz * sizeof(double), (on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice), s_));
        if (P_->assembled_len) SPAND_CUDA(cudaMemsetAsync(pristine_, 0, P_->assembled_len * sizeof(T), s_));
        if (nnz > 0) {
            assemble_scatter_kernel<T><<<(unsigned)((nnz + 255) / 256), 256, 0, s_>>>(d_vals_, d_amap_, nnz, pristine_);
            SPAND_CUDA(cudaGetLastError());
        }
        factored_ = false;
    }
    const double* device_values() const override { return d_vals_; }

    // factorize() as one CUDA graph: captured on the first factorization after the launch
    // configuration was tuned, replayed by every later one.  Every size lives in device
    // memory and the inputs are restored from the HBM-resident assembled blocks, so one
    // graph serves every re-factorization of the plan; it is captured again when the
    // tolerance (a kernel argument) or the preservation buffers change.  Profiled runs and
    // SPAND_CHECK_LAUNCHES run the launches one by one.
    void factorize_enqueue(double tol) override {
        last_tol_ = tol;
        if (tuned_ && tol != tuned_tol_) {
            // another tolerance changes every rank: this factorization runs launch by launch
            // on the current configuration (whose kernels take larger matrices on their
            // fallback paths) and the launches are tuned again from its sizes
            tuned_ = false;
            measure_next_ = false;
        }
        if (measure_next_) {
            // the factorization after tuning times the candidate QRCP launches per wave
            measure_next_ = false;
            measuring_ = true;
            enqueue_factor(tol);
            return;
        }
        const bool graphable = use_fgraph_ && tuned_ && !prof_.enabled() && !check_launches_;
        if (!graphable) {
            enqueue_factor(tol);
            return;
        }
        if (!fgraph_exec_ || fgraph_tol_ != tol || fgraph_nphi_ != nphi_) {
            drop_factor_graph();
            const int64_t before = launches_;
            SPAND_CUDA(cudaStreamBeginCapture(s_, cudaStreamCaptureModeThreadLocal));
            try {
                enqueue_factor(tol);
            } catch (...) {
                cudaGraph_t g = nullptr;
                cudaStreamEndCapture(s_, &g);
                if (g) cudaGraphDestroy(g);
                launches_ = before;
                throw;
            }
            SPAND_CUDA(cudaStreamEndCapture(s_, &fgraph_));
            SPAND_CUDA(cudaGraphInstantiate(&fgraph_exec_, fgraph_, 0));
            fgraph_kernels_ = launches_ - before;
            launches_ = before;
            fgraph_tol_ = tol;
            fgraph_nphi_ = nphi_;
        }
        SPAND_CUDA(cudaGraphLaunch(fgraph_exec_, s_));
        launches_ += fgraph_kernels_;
    }
    void drop_factor_graph() {
        if (fgraph_exec_) cudaGraphExecDestroy(fgraph_exec_);
        if (fgraph_) cudaGraphDestroy(fgraph_);
        fgraph_exec_ = nullptr;
        fgraph_ = nullptr;
    }
    int64_t factor_graph_kernels() const { return fgraph_exec_ ? fgraph_kernels_ : -1; }

    void enqueue_factor(double tol) {
        const Plan& P = *P_;
        gskip_used_ = false;
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
        pres_adaptive_ = nphi_ > 0 && tol <= 1.0;
        if (nphi_)
            launch("preserve_init", [&] {
                preserve_init<T>(phictx(), d_phinat_, phi_n_, d_perm_, d_phidst_, d_phild_, s_);
            });
        bool side_used = false;
        for (int l = 0; l < P.nlevels; l++) {
            LevelDev& D = levels_[l];
            cur_level_ = l;
            if (D.n_elim) {
                if (lu_) {
                    launch_getrf(D.elim_pivots, D.elim_inv, D.elim_clusters, D.n_elim, D.elim_lu_smem);
                    launch_lu_trsm(D.elim_trsm0);
                    launch_lu_trsm(D.elim_trsm1);
                } else if (ldlt_) {
                    launch_ldlt(D.elim_pivots, D.elim_clusters, nullptr, D.n_elim, D.elim_lu_smem);
                    launch_trsm(D.elim_trsm0);
                    launch_trsm(D.elim_trsm1);
                } else {
                    launch_potrf(D.elim_pivots, D.elim_clusters, D.n_elim, D.elim_ps_piv, D.elim_ps_cl, D.n_elim_ps,
                                 D.elim_pb_piv, D.elim_pb_cl, D.n_elim_pb,
                                 D.elim_smem, D.elim_tri, D.elim_pc_cs,
                                 D.elim_pc_smem, D.elim_split);
                    launch_trsm(D.elim_trsm0);
                    launch_trsm(D.elim_trsm1);
                }
                launch_schur(D.schur_targets, d_ups_, D.schur_tiles, D.n_schur_tiles);
            }
            if (D.scaled && D.n_scale) {
                scale_phase_ = true;
                if (lu_) {
                    launch_getrf(D.scale_pivots, D.scale_inv, D.scale_clusters, D.n_scale, D.scale_lu_smem);
                    launch_lu_trsm(D.scale_trsm0);
                    launch_lu_trsm(D.scale_trsm1);
                } else if (ldlt_) {
                    launch_ldlt(D.scale_pivots, D.scale_clusters, D.scale_newpiv, D.n_scale, D.scale_lu_smem);
                    launch_trsm(D.scale_trsm0);
                    launch_trsm(D.scale_trsm1);
                } else {
                    launch_potrf(D.scale_pivots, D.scale_clusters, D.n_scale, D.scale_ps_piv, D.scale_ps_cl,
                                 D.n_scale_ps, D.scale_pb_piv, D.scale_pb_cl, D.n_scale_pb, D.scale_smem, D.scale_tri,
                                 D.scale_pc_cs, D.scale_pc_smem, D.scale_split);
                    launch_trsm(D.scale_trsm0);
                    launch_trsm(D.scale_trsm1);
                    if (lorasp_)
                        launch("identity", [&] {
                            identity_kernel<T><<<D.n_scale, 128, 0, s_>>>(ctx_, D.scale_newpiv, D.scale_clusters);
                        });
                }
                if (nphi_)
                    launch("preserve_scale", [&] {
                        preserve_scale<T>(ctx_, phictx(), phitmp_, D.scale_clusters, D.scale_pivots, D.n_scale,
                                          ldlt_ ? lu_perm_ : nullptr, d_xoff_, s_);
                    });
                scale_phase_ = false;
            }
            if (D.n_level)
                launch("snapshot", [&] {
                    launch_pdl(snapshot_kernel, dim3((D.n_level + 255) / 256), dim3(256), 0, 1, (const int*)csize_,
                               rows0_, (const int*)D.level_clusters, D.n_level);
                });
            for (size_t wi = 0; wi < D.waves.size(); wi++) {
                WaveDev& W = D.waves[wi];
                if (nphi_) {
                    // preservation (tree.cpp:1257-1409): Q from [A_sn phi, phi] (and the QRCP
                    // of what it leaves of Asn), applied to phi and to every edge block
                    launch("preserve_basis", [&] {
                        preserve_basis<T>(ctx_, phictx(), W.items, W.n, pieces_, ldlt_ ? signs_ : nullptr, d_xoff_,
                                          vstore_, tauws_, rank1_, rank_, pres_adaptive_, s_);
                    });
                    if (pres_adaptive_) {
                        launch("qrcp", [&] { launch_qrcp_cluster(W, tol); });
                        launch("qrcp_global", [&] { launch_qrcp_global(W, tol); });
                        launch("preserve_combine", [&] {
                            preserve_combine<T>(ctx_, W.items, W.n, ws_, vstore_, tauws_, rank1_, rank_, s_);
                        });
                    }
                    // the WY factors first: the Q^T application uses them
                    launch("sparsify_wy", [&] {
                        sparsify_wy_kernel<T><<<W.n, 256, larft_smem_elems() * sizeof(T), s_>>>(
                            ctx_, W.items, vstore_, rank_, tauws_, taustore_, tstore_, ortho_full_on_ ? 1 : 0);
                    });
                    launch("preserve_apply", [&] {
                        preserve_apply<T>(ctx_, phictx(), W.items, W.n, W.ptiles, pieces_, vstore_, tstore_, rank_, s_);
                    });
                } else {
                    cur_wave_ = (int)wi;
                    launch("qrcp", [&] { launch_qrcp_cluster(W, tol); });
                    // matrices larger than the cluster's shared memory: the same algorithm with
                    // the slabs in global memory (clusters of other matrices exit at once).
                    // Not queued where the tuned launch holds every matrix of the wave at the
                    // sizes it was tuned for; a matrix that outgrew it raises the status's
                    // overflow flag and the factorization runs again with the pass queued.
                    if (!W.gskip) launch("qrcp_global", [&] { launch_qrcp_global(W, tol); });
                    gskip_used_ |= W.gskip;
                    launch("sparsify_scatter", [&] {
                        launch_pdl(sparsify_scatter_kernel<T>, dim3((unsigned)W.n, (unsigned)W.ytiles), dim3(256), 0, 1,
                                   ctx_, (const DSpars*)W.items, (const DAsn*)pieces_, (const T*)ws_,
                                   (const int*)ipvt_, (const int*)rank_, vstore_);
                    });
                }
                if (lorasp_) {
                    // Q^T on the original edges, their last rows to the siblings, then the
                    // siblings' elimination: Schur updates between their neighbours
                    launch("sparsify_wy", [&] {
                        sparsify_wy_kernel<T><<<W.n, 256, larft_smem_elems() * sizeof(T), s_>>>(
                            ctx_, W.items, vstore_, rank_, tauws_, taustore_, tstore_, ortho_full_on_ ? 1 : 0);
                    });
                    launch("lorasp_split", [&] {
                        lorasp_split<T>(ctx_, W.items, W.n, W.stiles, W.sib, W.orng, lr_splits_, vstore_, tstore_,
                                        rank_, s_);
                    });
                    launch_schur(D.schur_targets, d_ups_, D.schur_tiles, D.n_schur_tiles);
                }
                if (ldlt_) {
                    launch("pivot_split", [&] {
                        pivot_split_kernel<T><<<W.n, 256, 0, s_>>>(ctx_, W.items, W.sib, W.sib_piv, W.aso, W.piv,
                                                                  vstore_, tauws_, signs_, d_xoff_);
                    });
                    launch_ldlt(W.sib_piv, W.sib, nullptr, W.n, W.ldlt_smem);
                    launch_trsm(W.sib_trsm);
                    launch_schur(W.sib_targets, W.sib_ups, W.sib_tiles, W.n_sib_tiles);
                }
                cur_wave_ = -1;
                // WY factors: on the side stream beside the next wave's QRCP (on the main
                // stream when the profiler times every launch); preservation and LoRaSp made
                // them above
                if (nphi_ || lorasp_) {
                } else if (prof_.enabled() || check_launches_) {
                    launch("sparsify_wy", [&] {
                        sparsify_wy_kernel<T><<<W.n, 256, larft_smem_elems() * sizeof(T), s_>>>(
                            ctx_, W.items, vstore_, rank_, tauws_, taustore_, tstore_, ortho_full_on_ ? 1 : 0);
                    });
                } else {
                    SPAND_CUDA(cudaEventRecord(ev_fork_, s_));
                    SPAND_CUDA(cudaStreamWaitEvent(s2_, ev_fork_, 0));
                    sparsify_wy_kernel<T><<<W.n, 256, larft_smem_elems() * sizeof(T), s2_>>>(
                        ctx_, W.items, vstore_, rank_, tauws_, taustore_, tstore_, ortho_full_on_ ? 1 : 0);
                    launches_ += 1;
                    side_used = true;
                }
            }
            if (D.merged && D.n_parents) {
                launch("merge_sizes", [&] {
                    launch_pdl(merge_sizes_kernel, dim3((D.n_parents + 127) / 128), dim3(128), 0, 1, csize_, rows0_,
                               cpos_, (const int*)D.parents, D.n_parents, (const int*)D.child_ptr,
                               (const int*)D.child_idx);
                });
                if (D.n_merge_tiles)
                    launch("merge_copy", [&] {
                        launch_pdl(merge_copy_kernel<T>, dim3(D.n_merge_tiles), dim3(256), 0, 1, ctx_,
                                   (const DMerge*)D.merge_items, (const DTile*)D.merge_tiles, D.n_merge_tiles,
                                   (const int*)cpos_);
                    });
                if (nphi_)
                    launch("preserve_merge", [&] {
                        preserve_merge<T>(ctx_, phictx(), D.parents, D.n_parents, D.child_ptr, D.child_idx, cpos_,
                                          s_);
                    });
            }
        }
        cur_level_ = -1;
        if (side_used) {
            SPAND_CUDA(cudaEventRecord(ev_join_, s2_));
            SPAND_CUDA(cudaStreamWaitEvent(s_, ev_join_, 0));
        }
        SPAND_CUDA(cudaGetLastError());
        if (!h_status_) SPAND_CUDA(cudaMallocHost(&h_status_, sizeof(DStatus)));
        SPAND_CUDA(cudaMemcpyAsync(h_status_, status_, sizeof(DStatus), cudaMemcpyDeviceToHost, s_));
    }

    void factorize_finish() override {
        SPAND_CUDA(cudaStreamSynchronize(s_));
        const DStatus st = *h_status_;
        if (st.overflow && gskip_used_) {
            // a matrix outgrew the tuned launch of its wave and its global-memory pass was not
            // queued: everything after it is void; factor again with every pass queued
            for (LevelDev& D : levels_)
                for (WaveDev& W : D.waves) W.gskip = false;
            drop_factor_graph();
            factorize_enqueue(last_tol_);
            factorize_finish();
            return;
        }
        failed_cluster_ = st.not_spd - 1;
        if (st.not_spd)
            throw DeviceError{SPAND_ERR_NOT_SPD, std::string(lu_ || ldlt_ ? "Error: Singular Pivot" : "Error: Non-SPD Pivot") +
                                                     " (cluster " + std::to_string(st.not_spd - 1) + ")"};
        factored_ = true;
        if (measuring_) {
            measuring_ = false;
            std::vector<QcConf> chosen;
            for (LevelDev& D : levels_)
                for (WaveDev& W : D.waves) chosen.push_back(QcConf{W.rpl, W.cs, W.threads, W.smem, W.vec_rows, 0.0});
            std::lock_guard<std::mutex> lk(qc_tune_mutex());
            qc_tune_cache()[tune_key_] = chosen;
        }
        if (!tuned_) tune_qrcp();
    }

    // Size the QRCP clusters of every wave from the matrices of the last factorization
    // (10% slack); a later factorization whose matrices outgrow them takes the fallback.
    void tune_qrcp() {
        std::vector<int> cs, r0;
        sizes(cs, r0);
        if (relayer_on_ && !ldlt_ && !lorasp_ && !nphi_ && !phi_alloc_) relayer_waves(cs, r0);
        {
            char buf[96];
            snprintf(buf, sizeof(buf), "T%d|sm%d|tol%a|", (int)sizeof(T), num_sms_, last_tol_);
            tune_key_ = buf;
        }
        tuned_tol_ = last_tol_;
        for (LevelDev& D : levels_) {
            std::map<int, int> wave_of;
            for (size_t w = 0; w < D.waves.size(); w++)
                for (const SparsifyItem& it : D.waves[w].host) wave_of[it.cluster] = (int)w;
            for (size_t w = 0; w < D.waves.size(); w++) {
                std::vector<std::pair<int, int>> dims;
                for (const SparsifyItem& it : D.waves[w].host) {
                    int64_t cols = 0;
                    for (int p = 0; p < it.count; p++) {
                        int n = P_->asn_pieces[it.first + p].nbr;
                        auto wn = wave_of.find(n);
                        cols += (wn != wave_of.end() && wn->second < (int)w) ? cs[n] : r0[n];
                    }
                    // 10% slack for the sizes of later factorizations
                    int rows = r0[it.cluster];
                    dims.push_back({rows + rows / 10 + 1, (int)(cols + cols / 10 + 1)});
                }
                choose_cluster(D.waves[w], dims, measure_on_);
                tune_key_ += std::to_string(D.waves[w].n) + ":";
                for (const auto& d : dims) tune_key_ += std::to_string(d.first) + "x" + std::to_string(d.second) + ",";
                tune_key_ += ";";
                if (per_wave_) {
                    int maxr = 0;
                    for (const SparsifyItem& it : D.waves[w].host) maxr = std::max(maxr, r0[it.cluster]);
                    const WaveDev& Wv = D.waves[w];
                    fprintf(stderr, "qrcp wave L%d w%zu: items %d max rows %d rpl %d cs %d threads %d smem %d active %d\n",
                            (int)(&D - levels_.data()), w, Wv.n, maxr, Wv.rpl, Wv.cs, Wv.threads, Wv.smem,
                            active_clusters(Wv.n * Wv.cs, Wv.cs, Wv.smem, Wv.threads,
                                            Wv.rpl ? qrcp_blocked_kernel_ptr<T>(Wv.rpl) : qrcp_smem_kernel_ptr<T>(Wv.threads)));
                }
            }
        }
        // POTRF / TRSM shared memory from the actual pivot sizes (10% slack; larger
        // pivots in a later factorization take the global-memory branch of the kernels)
        for (size_t l = 0; l < levels_.size(); l++) {
            LevelDev& D = levels_[l];
            const LevelPlan& L = P_->levels[l];
            auto nmax = [&](const std::vector<int>& cl) {
                int m = 0;
                for (int c0 : cl) m = std::max(m, r0[c0]);
                return m + m / 10 + 1;
            };
            int ne = nmax(L.elim_clusters), ns = nmax(L.scale_clusters);
            D.elim_smem = potrf_smem_n(ne);
            D.scale_smem = potrf_smem_n(ns);
            D.elim_split = potrf_split_pays(L.elim_clusters, r0, D.elim_smem);
            D.scale_split = potrf_split_pays(L.scale_clusters, r0, D.scale_smem);
            choose_potrf_cluster(ne, D.elim_smem, D.n_elim, D.elim_pc_cs, D.elim_pc_smem);
            choose_potrf_cluster(ns, D.scale_smem, D.n_scale, D.scale_pc_cs, D.scale_pc_smem);
            // the strip inverse must take every pivot the cluster Cholesky holds: its shared
            // memory, rounded up to 256 bytes, admits pivots up to one row above nmax
            D.elim_tri.smem = trtri_smem_n(ne + 2);
            D.scale_tri.smem = trtri_smem_n(ns + 2);
            if (!ldlt_) {  // the LDLT panels always stage: keep their capacity-sized buffers
                D.elim_trsm0.smem = D.elim_trsm1.smem = trsm_smem_n(ne);
                D.scale_trsm0.smem = D.scale_trsm1.smem = trsm_smem_n(ns);
            }
        }
        tuned_ = true;
        // configurations measured before for the same plan, sizes, tolerance and GPU: no
        // measuring factorization
        measure_next_ = false;
        if (measure_on_) {
            std::lock_guard<std::mutex> lk(qc_tune_mutex());
            auto hit = qc_tune_cache().find(tune_key_);
            if (hit != qc_tune_cache().end() && hit->second.size() == n_waves()) {
                size_t k = 0;
                for (LevelDev& D : levels_)
                    for (WaveDev& W : D.waves) apply_conf(W, hit->second[k++]);
            } else {
                for (LevelDev& D : levels_)
                    for (WaveDev& W : D.waves) measure_next_ |= W.cands.size() > 1;
            }
        }
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

    void set_phi(const double* phi, int n, int nphi) override {
        if (nphi <= 0) {
            nphi_ = 0;
            return;
        }
        const Plan& P = *P_;
        if (n != (int)perm_h_.size()) throw DeviceError{SPAND_ERR_ARG, "phi does not match the matrix size"};
        long long capsum = 0;
        for (int c0 = 0; c0 < P.nclusters_h; c0++) capsum += P.c_cap[c0];
        if (nphi > phi_alloc_ || !rank1_ || nphi != nphi_ || !d_phioff_) drop_factor_graph();  // buffers change
        if (nphi > phi_alloc_) {
            phis_ = alloc<T>(capsum * nphi);
            phitmp_ = alloc<T>(capsum * nphi);
            d_phinat_ = alloc<double>((int64_t)n * nphi);
            phi_alloc_ = nphi;
        }
        if (!rank1_) rank1_ = alloc<int>(nc_);
        if (nphi != nphi_ || !d_phioff_) {
            std::vector<long long> off(nc_, 0), dst(std::max(n, 1), 0);
            std::vector<int> ld(std::max(n, 1), 1);
            long long o = 0;
            for (int c0 = 0; c0 < P.nclusters_h; c0++) {
                off[c0] = o;
                o += (long long)P.c_cap[c0] * nphi;
            }
            for (int c0 = 0; c0 < P.nclusters_h; c0++)
                if (P.c_hlevel[c0] == 0)
                    for (int i = 0; i < P.c_cap[c0]; i++) {
                        dst[P.c_start[c0] + i] = off[c0] + i;
                        ld[P.c_start[c0] + i] = P.c_cap[c0];
                    }
            d_phioff_ = up(off);
            d_phidst_ = up(dst);
            d_phild_ = up(ld);
            for (auto& D : levels_)
                for (auto& W : D.waves) {
                    W.ptiles = 1;
                    for (const SparsifyItem& it : W.host) {
                        std::vector<int> caps;
                        for (int p = 0; p < it.count; p++) caps.push_back(P.c_cap[P.asn_pieces[it.first + p].nbr]);
                        W.ptiles = std::max(W.ptiles, preserve_apply_tiles(caps.data(), it.count, nphi));
                    }
                }
        }
        nphi_ = nphi;
        phi_n_ = n;
        if (n > 0)
            SPAND_CUDA(cudaMemcpyAsync(d_phinat_, phi, (size_t)n * nphi * sizeof(double), cudaMemcpyHostToDevice, s_));
        SPAND_CUDA(cudaStreamSynchronize(s_));
        factored_ = false;
    }

    void solve_device_noalloc(double* x, int nrhs, int ld) override {
        if (!factored_) throw DeviceError{SPAND_ERR_STATE, "solve before factorize"};
        const size_t need = 2 * (size_t)xld_ * (size_t)nrhs * sizeof(T);
        if (need > kNoAllocSolveScratchBytes)
            throw DeviceError{SPAND_ERR_ARG, "allocation-free solve needs " + std::to_string(need) +
                                                 " bytes of solve vectors and their scratch copy (2 x " +
                                                 std::to_string(xld_) + " x " + std::to_string(nrhs) + " x " +
                                                 std::to_string(sizeof(T)) + "); its fixed scratch holds " +
                                                 std::to_string(kNoAllocSolveScratchBytes) + " bytes"};
        T* slots = static_cast<T*>(noalloc_solve_scratch(dev_));
        const bool was_on = prof_.enabled();  // the profiler creates CUDA events
        prof_.enable(false);
        try {
            run_solve_slots(x, nrhs, ld, slots, slots + (size_t)xld_ * nrhs);
        } catch (...) {
            prof_.enable(was_on);
            throw;
        }
        prof_.enable(was_on);
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

    void ldlt_signs(int cl, std::vector<double>& out) override {
        std::vector<T> t(P_->c_cap[cl], T(0));
        if (signs_ && !t.empty()) {
            SPAND_CUDA(cudaMemcpyAsync(t.data(), signs_ + P_->c_xoff[cl], t.size() * sizeof(T), cudaMemcpyDeviceToHost,
                                       s_));
            SPAND_CUDA(cudaStreamSynchronize(s_));
        }
        out.assign(t.begin(), t.end());
    }

    void lu_perm(int cl, std::vector<int>& out) override {
        out.assign(P_->c_cap[cl], 0);
        if (!lu_perm_ || out.empty()) return;
        SPAND_CUDA(cudaMemcpyAsync(out.data(), lu_perm_ + P_->c_xoff[cl], out.size() * sizeof(int),
                                   cudaMemcpyDeviceToHost, s_));
        SPAND_CUDA(cudaStreamSynchronize(s_));
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
        int smem = 0;
        // the same tiles split by pivot size: at most 32 rows (a warp each on the tensor
        // cores, FP32) and larger
        DTile* stiles = nullptr;
        int nstiles = 0;
        DTile* btiles = nullptr;
        int nbtiles = 0;
    };
    struct TrtriDev {
        DTile* tiles = nullptr;
        int ntiles = 0;
        int smem = 0;
    };
    // one launch configuration of a wave's shared-memory QRCP (rpl 0: the unblocked kernel)
    struct QcConf {
        int rpl = 0, cs = 1, threads = QC_THREADS, smem = 0;
        int vec_rows = INT_MAX;  // slabs of at least this many rows: vectorised trailing update
        double est = 0.0;  // the launch model's estimate (arbitrary units)
    };
    struct WaveDev {
        int n = 0;
        DSpars* items = nullptr;
        int maxcap = 1;
        std::vector<QcConf> cands;  // launch configurations the measuring factorization times
        std::vector<std::pair<QcConf, float>> timed;  // what it measured (ms per candidate)
        bool gskip = false;  // tuned launch holds every matrix: no global-memory pass queued
        int64_t cols = 0;           // Asn columns of all its matrices (pivot workspace)
        int rpl = 0;         // > 0: the blocked QRCP for up to 32 * rpl rows; 0: the unblocked kernel
        int vec_rows = INT_MAX;  // unblocked kernel: slabs of at least this many rows are vectorised
        int cs = 1;          // CTAs per thread-block cluster of the shared-memory QRCP
        int threads = QC_THREADS;  // threads per CTA of that launch
        int smem = 0;        // dynamic shared memory per CTA
        int gcs = 1;         // cluster of the global-memory QRCP (matrices the first does not hold)
        int gsmem = 0;       // its dynamic shared memory per CTA
        int ytiles = 0;      // scatter tiles per matrix (reflector + edge-block capacity tiles)
        int ptiles = 0;      // preservation: Q^T-application CTAs per matrix
        int2* orng = nullptr;  // LoRaSp: per item its slice of the original edges
        int stiles = 0;        // LoRaSp: split CTAs per matrix
        // LDLT: per item the sibling, its pivot, the edge block, the cluster's pivot; the
        // sibling panels and the Schur update of the cluster's pivot
        int *sib = nullptr, *sib_piv = nullptr, *aso = nullptr, *piv = nullptr;
        TrsmDev sib_trsm;
        DTarget* sib_targets = nullptr;
        DUpd* sib_ups = nullptr;
        DTile* sib_tiles = nullptr;
        int n_sib_tiles = 0, ldlt_smem = 0;
        std::vector<SparsifyItem> host;  // plan items, for tuning
    };
    struct LevelDev {
        int n_elim = 0;
        int* elim_clusters = nullptr;
        int* elim_pivots = nullptr;
        int *elim_ps_cl = nullptr, *elim_ps_piv = nullptr, *scale_ps_cl = nullptr, *scale_ps_piv = nullptr;
        int n_elim_ps = 0, n_scale_ps = 0;  // LLT pivots of at most 32 rows (a warp each)
        int *elim_pb_cl = nullptr, *elim_pb_piv = nullptr, *scale_pb_cl = nullptr, *scale_pb_piv = nullptr;
        int n_elim_pb = 0, n_scale_pb = 0;  // the other LLT pivots
        int elim_smem = 0;
        int elim_pc_cs = 0, elim_pc_smem = 0;   // cluster Cholesky (0: single-CTA kernel)
        bool elim_split = false;                 // one-CTA Cholesky launched per size class
        TrsmDev elim_trsm0, elim_trsm1;
        TrtriDev elim_tri, scale_tri;
        DTarget* schur_targets = nullptr;
        DTile* schur_tiles = nullptr;
        int n_schur_tiles = 0;
        bool scaled = false;
        int n_scale = 0;
        int* scale_clusters = nullptr;
        int* scale_pivots = nullptr;
        int scale_smem = 0;
        int scale_pc_cs = 0, scale_pc_smem = 0;
        bool scale_split = false;
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
        // many right-hand sides: small clusters (indices into the op lists) and the row tiles
        // of the others
        int *elim_small = nullptr, *scale_small = nullptr;
        int n_elim_small = 0, n_scale_small = 0;
        int2 *elim_big_tv = nullptr, *scale_big_tv = nullptr;
        int n_elim_big_tv = 0, n_scale_big_tv = 0;
        int *elim_inv = nullptr, *scale_inv = nullptr;  // PLU: inverse blocks, parallel to the pivots
        int elim_lu_smem = 0, scale_lu_smem = 0;
        // LDLT: new sign pivots of the scaled clusters; siblings of the sparsified clusters
        // (solve lists: their pivots, trsv tiles, GemmSymmIn groups forward by cluster and
        // backward by sibling)
        int* scale_newpiv = nullptr;
        int n_sib = 0, n_sib_tv = 0, x_smem_sib = 0;
        int *sib_clusters = nullptr, *sib_owner = nullptr, *sib_piv = nullptr;
        int2* sib_tv = nullptr;
        DGroup *sib_gf = nullptr, *sib_gb = nullptr;
        DGemmOp *sib_gfo = nullptr, *sib_gbo = nullptr;
        DTile *sib_gf_tiles = nullptr, *sib_gb_tiles = nullptr;
        int n_sib_gf_tiles = 0, n_sib_gb_tiles = 0;
        int *elim_llt = nullptr, *elim_llt_blk = nullptr, *scale_llt = nullptr, *scale_llt_blk = nullptr;
        int x_smem_elim = 0, x_smem_scale = 0, x_smem_ortho = 0;
        DTile* gf_tiles32 = nullptr;  // forward Gemm groups in 32-row tiles (many right-hand sides)
        int n_gf_tiles32 = 0;
        int ortho_mrhs_smem = 0;      // x of 32 right-hand sides (rows x 33); 0: one at a time
        int ortho_full_smem = 0;      // the whole-T Orthogonal op's x, w, y (0: too large, blocked form)
        bool ortho_full_wide = false; // its 512-thread instantiation (clusters of 96 rows or more)
        int ortho_cs = 1;             // > 1: the thread-block-cluster form, CTAs per cluster
        int ortho_cs_smem = 0;        // its shared memory
        int2 *elim_tv = nullptr, *scale_tv = nullptr;  // (item, row tile) of the triangular products
        int n_elim_tv = 0, n_scale_tv = 0;
        int n_gf = 0, n_gb = 0;
        DGroup *gf = nullptr, *gb = nullptr;
        DTile *gf_tiles = nullptr, *gb_tiles = nullptr;
        int n_gf_tiles = 0, n_gb_tiles = 0;
        DGemmOp *gfo = nullptr, *gbo = nullptr;
        int n_ortho = 0;
        DOrtho* ortho = nullptr;
    };

    // The device record of a sparsification wave (the matrices' work list, scatter tiles, the
    // launch from capacity bounds and the global-memory fallback's launch); the wave's items
    // carry their workspace offsets.  Workspaces grow here when a wave needs more.
    WaveDev make_wave(const std::vector<SparsifyItem>& wave) {
        const Plan& P = *P_;
        WaveDev W;
        std::vector<DSpars> items;
        int64_t coloff = 0, ws = 0;
        int maxcap = 1;
        for (const SparsifyItem& it : wave) {
            items.push_back({it.cluster, it.first, it.count, it.cap_cols, (long long)it.ws_off, (long long)coloff,
                             (long long)it.v_off, (long long)it.tau_off});
            coloff += std::max(it.cap_cols, 1);
            maxcap = std::max(maxcap, P.c_cap[it.cluster]);
            ws = std::max<int64_t>(ws, it.ws_off + (int64_t)P.c_cap[it.cluster] * std::max(it.cap_cols, 1));
        }
        W.cols = coloff;
        W.n = (int)items.size();
        W.items = up(items);
        W.maxcap = maxcap;
        W.ytiles = 1;  // capacities can be 0 (LoRaSp bounds): never an empty grid
        for (const SparsifyItem& it : wave) {
            int nt = (P.c_cap[it.cluster] + 31) / 32;
            for (int p = 0; p < it.count; p++) nt += (P.c_cap[P.asn_pieces[it.first + p].nbr] + 31) / 32;
            W.ytiles = std::max(W.ytiles, nt);
        }
        W.host = wave;
        // capacity bound until the first factorization reports the actual sizes
        std::vector<std::pair<int, int>> dims;
        for (const SparsifyItem& it : wave) dims.push_back({P.c_cap[it.cluster], it.cap_cols});
        choose_cluster(W, dims);
        // global-memory launch: a full cluster where some matrix at its capacity could exceed
        // the largest shared-memory configuration, else one CTA as the safety net for sizes
        // that grow beyond the tuned configuration
        bool big = false;
        for (const auto& d : dims) big |= qc_need(d.first, d.second, qc_max_cs_, (int)sizeof(T)) > qc_smem_cap_;
        W.gcs = (big || force_global_) ? qc_max_cs_ : 1;
        int64_t g = 4096;
        for (const auto& d : dims) g = std::max<int64_t>(g, qc_small_need(d.first, d.second, W.gcs, (int)sizeof(T)));
        if (g > qc_smem_cap_) throw DeviceError{SPAND_ERR_UNSUPPORTED, "sparsification matrix too large for the QRCP kernels"};
        W.gsmem = (int)((g + 255) & ~int64_t(255));
        // workspaces of a re-layered wave (the plan sized them for its own waves)
        if (ws_ && ws > ws_len_) {
            ws_ = alloc<T>(ws);
            ws2_ = alloc<T>(ws);
            ws_len_ = ws;
        }
        if (jpvt_ && coloff > cols_len_) {
            jpvt_ = alloc<int>(coloff);
            ipvt_ = alloc<int>(coloff);
            cols_len_ = coloff;
        }
        if (fallback_ && W.n > items_len_) {
            fallback_ = alloc<int>(W.n);
            colcount_ = alloc<int>(W.n);
            items_len_ = W.n;
        }
        return W;
    }

    // Re-layer a level's sparsification into waves that fill the GPU (plain path, levels of
    // small matrices: clusters of at most 4 CTAs).  A matrix depends only on its neighbours
    // sparsified before it (they rewrote the edge blocks it gathers); the plan's waves put
    // each matrix one wave after its latest such neighbour, however many matrices a wave
    // then holds, so a wave of N matrices on A co-resident clusters ends with a partly
    // filled round while later matrices that do not depend on its last ones wait.  With the
    // actual sizes known, list scheduling builds waves of at most A matrices (A: co-resident clusters of the level's launch configuration), each
    // matrix placed after all its dependencies, the ready matrices with the longest chains of
    // dependents first; inside a wave the largest matrices start first.  Any order that keeps
    // every dependency gives the same gathers and the same results bit for bit.
    void relayer_waves(const std::vector<int>& cs, const std::vector<int>& r0) {
        const Plan& P = *P_;
        for (LevelDev& D : levels_) {
            std::vector<SparsifyItem> items;
            std::vector<int> owave;
            for (size_t w = 0; w < D.waves.size(); w++)
                for (const SparsifyItem& it : D.waves[w].host) {
                    items.push_back(it);
                    owave.push_back((int)w);
                }
            const int n = (int)items.size();
            if (n < 2) continue;
            std::map<int, int> idx_of;
            for (int i = 0; i < n; i++) idx_of[items[i].cluster] = i;
            std::vector<std::vector<int>> deps(n), users(n);
            std::vector<std::pair<int, int>> dims(n);
            std::vector<double> work(n);
            for (int i = 0; i < n; i++) {
                const SparsifyItem& it = items[i];
                int64_t cols = 0;
                for (int p = 0; p < it.count; p++) {
                    const int nb = P.asn_pieces[it.first + p].nbr;
                    auto f = idx_of.find(nb);
                    const bool before = f != idx_of.end() && owave[f->second] < owave[i];
                    cols += before ? cs[nb] : r0[nb];
                    if (before) {
                        deps[i].push_back(f->second);
                        users[f->second].push_back(i);
                    }
                }
                const int rows = r0[it.cluster];
                dims[i] = {rows + rows / 10 + 1, (int)(cols + cols / 10 + 1)};
                work[i] = (double)rows * (double)cols;
            }
            // co-resident clusters of the launch the level's matrices would take together
            WaveDev probe;
            probe.n = n;
            choose_cluster(probe, dims, false, false);  // the same waves whatever is forced
            const QcKernel<T> fn =
                probe.rpl > 0 ? qrcp_blocked_kernel_ptr<T>(probe.rpl) : qrcp_smem_kernel_ptr<T>(probe.threads);
            // Levels whose matrices need clusters of 8 or 16 CTAs keep their waves: with so few
            // co-resident clusters the new waves are one round each and lose the overlap of
            // uneven matrices inside a larger launch (measured slower at 64^3, levels 4-7).
            if (probe.cs > 4) continue;
            const int A = std::max(1, active_clusters(probe.n * probe.cs, probe.cs, probe.smem, probe.threads, fn));
            // longest chain of dependents (items are in a dependency order: waves ascending)
            std::vector<int> height(n, 1);
            for (int i = n - 1; i >= 0; i--)
                for (int u : users[i]) height[i] = std::max(height[i], height[u] + 1);
            std::vector<int> layer(n, -1), left(n);
            for (int i = 0; i < n; i++) left[i] = (int)deps[i].size();
            std::vector<int> ready;
            for (int i = 0; i < n; i++)
                if (!left[i]) ready.push_back(i);
            std::vector<std::vector<int>> layers;
            int placed = 0;
            while (placed < n) {
                std::stable_sort(ready.begin(), ready.end(), [&](int a, int b) {
                    return height[a] != height[b] ? height[a] > height[b] : work[a] > work[b];
                });
                const int take = std::min<int>(A, (int)ready.size());
                std::vector<int> cur(ready.begin(), ready.begin() + take);
                ready.erase(ready.begin(), ready.begin() + take);
                for (int i : cur) layer[i] = (int)layers.size();
                for (int i : cur)
                    for (int u : users[i])
                        if (--left[u] == 0) ready.push_back(u);
                placed += take;
                std::stable_sort(cur.begin(), cur.end(), [&](int a, int b) { return work[a] > work[b]; });
                layers.push_back(cur);
            }
            std::vector<WaveDev> waves;
            for (const auto& lay : layers) {
                std::vector<SparsifyItem> wave;
                int64_t ws = 0;
                for (int i : lay) {
                    SparsifyItem it = items[i];
                    it.ws_off = ws;
                    ws += (int64_t)P.c_cap[it.cluster] * std::max(it.cap_cols, 1);
                    ws = (ws + 31) & ~int64_t(31);
                    wave.push_back(it);
                }
                waves.push_back(make_wave(wave));
            }
            D.waves.swap(waves);
        }
    }


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
        if (prof_.enabled() && per_level_ && cur_level_ >= 0) {
            std::string name = std::string(cls) + (scale_phase_ ? "@S" : "@L") + std::to_string(cur_level_);
            if (per_wave_ && cur_wave_ >= 0) name += "w" + std::to_string(cur_wave_);
            prof_.begin(s_, name.c_str());
        } else {
            prof_.begin(s_, cls);
        }
        f();
        if (check_launches_) {
            // SPAND_CHECK_LAUNCHES=1: name the launch that failed (with a wait after every
            // launch, so that a fault in the kernel itself is attributed to it too)
            cudaError_t e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaStreamSynchronize(s_);
            if (e != cudaSuccess)
                throw DeviceError{SPAND_ERR_CUDA, std::string(cls) + " (level " + std::to_string(cur_level_) +
                                                      ", wave " + std::to_string(cur_wave_) + "): " +
                                                      cudaGetErrorString(e)};
        }
        prof_.end(s_);
        launches_ += kernels;
    }
    void ensure_x(int nrhs) {
        if (nrhs <= x_nrhs_) return;
        if (xs_) cudaFree(xs_);
        xs_ = nullptr;
        // solve vectors and their scratch copy (second half)
        SPAND_CUDA(cudaMalloc(&xs_, 2 * (size_t)xld_ * nrhs * sizeof(T)));
        x_nrhs_ = nrhs;
    }
    int smem_for(const std::vector<int>& clusters, const Plan& P) {
        int mx = 0;
        for (int c0 : clusters) mx = std::max(mx, P.c_cap[c0]);
        return potrf_smem_n(mx);
    }
    int xsmem_for(const std::vector<int>& clusters, const Plan& P) {
        int mx = 1;
        for (int c0 : clusters) mx = std::max(mx, P.c_cap[c0]);
        const int64_t b = ((int64_t)mx + (TV_THREADS / 32) * 2 * TV_ROWS) * (int64_t)sizeof(T);
        if (b > 200 * 1024) throw DeviceError{SPAND_ERR_UNSUPPORTED, "cluster too large for the solve kernels"};
        return (int)b;
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
        auto t0 = tiles_1d(ext0, TRB);
        auto t1 = tiles_1d(ext1, TRB);
        side0 = {up(it0), up(t0), (int)t0.size(), 0, trsm_smem(clusters, P)};
        side1 = {up(it1), up(t1), (int)t1.size(), 1, trsm_smem(clusters, P)};
        auto split = [&](const std::vector<DTrsm>& it, const std::vector<DTile>& tl, TrsmDev& d) {
            std::vector<DTile> sm, bg;
            for (const DTile& x : tl) (P.c_cap[it[x.item].cluster] <= 32 ? sm : bg).push_back(x);
            d.stiles = up(sm);
            d.nstiles = (int)sm.size();
            d.btiles = up(bg);
            d.nbtiles = (int)bg.size();
        };
        split(it0, t0, side0);
        split(it1, t1, side1);
    }
    // ---- QRCP launch configuration -------------------------------------------------
    int qc_smem_cap_ = 0;  // dynamic shared memory per CTA available to the QRCP kernel
    int pc_smem_cap_ = 0;  // the same for the cluster Cholesky
    int qc_max_cs_ = 8;    // largest cluster (16 where non-portable sizes are allowed)
    int qb_smem_cap_ = 0;  // the same for the blocked QRCP kernels
    int qcw_smem_cap_ = 0;  // and for the wide (512-thread) unblocked QRCP
    int num_sms_ = 1;
    void init_qrcp_limits() {
        int dev = 0, optin = 0;
        SPAND_CUDA(cudaGetDevice(&dev));
        SPAND_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        SPAND_CUDA(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, dev));
        const QcKernel<T> fn = qrcp_smem_kernel_ptr<T>();
        cudaFuncAttributes fa;
        SPAND_CUDA(cudaFuncGetAttributes(&fa, fn));
        qc_smem_cap_ = (int)(optin - (int)fa.sharedSizeBytes) & ~255;
        SPAND_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, qc_smem_cap_));
        {
            cudaFuncAttributes pa;
            SPAND_CUDA(cudaFuncGetAttributes(&pa, potrf_cluster_kernel<T>));
            pc_smem_cap_ = (int)(optin - (int)pa.sharedSizeBytes) & ~255;
        }
        SPAND_CUDA(cudaFuncSetAttribute(potrf_cluster_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        pc_smem_cap_));
        SPAND_CUDA(cudaFuncSetAttribute(qrcp_gslab_kernel_ptr<T>(), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        qc_smem_cap_));
        if (cudaFuncSetAttribute(qrcp_gslab_kernel_ptr<T>(), cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
            cudaSuccess)
            cudaGetLastError();
        if (cudaFuncSetAttribute(potrf_cluster_kernel<T>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
            cudaSuccess)
            cudaGetLastError();
        qc_max_cs_ = 8;
        if (cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
            if (active_clusters(16, 16, qc_smem_cap_) > 0) qc_max_cs_ = 16;
        } else {
            cudaGetLastError();
        }
        // the wide unblocked QRCP (512 threads): its own cap (larger static arrays)
        {
            const QcKernel<T> wfn = qrcp_smem_kernel_ptr<T>(QC_WIDE_THREADS);
            SPAND_CUDA(cudaFuncGetAttributes(&fa, wfn));
            qcw_smem_cap_ = (int)(optin - (int)fa.sharedSizeBytes) & ~255;
            SPAND_CUDA(cudaFuncSetAttribute(wfn, cudaFuncAttributeMaxDynamicSharedMemorySize, qcw_smem_cap_));
            if (qc_max_cs_ > 8 && cudaFuncSetAttribute(wfn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
                cudaGetLastError();
        }
        // the blocked QRCP: every row-count instantiation gets the largest dynamic shared
        // memory its static arrays leave (the smallest of them is the cap) and, like the
        // unblocked kernel, non-portable cluster sizes
        qb_smem_cap_ = qc_smem_cap_;
        for (int rpl : {1, 2, 4, 8, 12}) {
            const QcKernel<T> b = qrcp_blocked_kernel_ptr<T>(rpl);
            SPAND_CUDA(cudaFuncGetAttributes(&fa, b));
            qb_smem_cap_ = std::min(qb_smem_cap_, (int)(optin - (int)fa.sharedSizeBytes) & ~255);
        }
        for (int rpl : {1, 2, 4, 8, 12}) {
            const QcKernel<T> b = qrcp_blocked_kernel_ptr<T>(rpl);
            SPAND_CUDA(cudaFuncSetAttribute(b, cudaFuncAttributeMaxDynamicSharedMemorySize, qb_smem_cap_));
            if (qc_max_cs_ > 8 && cudaFuncSetAttribute(b, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
                cudaGetLastError();
        }
    }
    // rows-per-lane instantiation of the blocked QRCP for matrices of up to `rows` rows (0: none)
    static int qb_rpl(int rows) {
        for (int r : {1, 2, 4, 8, 12})
            if (rows <= 32 * r) return r;
        return 0;
    }
    // co-resident thread-block clusters of a QRCP configuration (-1: not launchable)
    int active_clusters(int ctas, int cs, int smem, int threads = QC_THREADS, QcKernel<T> fn = nullptr) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)ctas);
        cfg.blockDim = dim3((unsigned)threads);
        cfg.dynamicSmemBytes = (size_t)smem;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)cs;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int n = -1;
        if (cudaOccupancyMaxActiveClusters(&n, fn ? fn : qrcp_smem_kernel_ptr<T>(), &cfg) != cudaSuccess) {
            cudaGetLastError();
            n = -1;
        }
        return n;
    }
    // Cluster size, threads per CTA and shared memory of a wave's QRCP launch.  dims:
    // (rows, cols) bound of every matrix of the wave.  Per candidate (cluster size, threads):
    // the slab of the largest matrix sets the shared memory, the occupancy query the number
    // of co-resident clusters (the kernel's registers cap a 256-thread CTA at two per SM;
    // 64-thread CTAs fit eight, which the many small matrices of the lower levels use); the
    // estimate is rounds x (per-step latency + passes over the largest slab by the CTA's
    // threads) and the smallest wins.
    void choose_cluster(WaveDev& W, const std::vector<std::pair<int, int>>& dims, bool collect = false,
                        bool honour_force = true) {
        double best = 1e300;
        int bcs = 0, bsm = 0, bth = QC_THREADS, bvec = INT_MAX;
        std::vector<QcConf> all;  // every launchable configuration with its estimate
        int maxrows_ = 0;
        for (const auto& d : dims) maxrows_ = std::max(maxrows_, d.first);
        // SPAND_QC_VEC=0 / 1: never / always (where the slabs are tall enough) the vectorised update
        const int force_vec = (honour_force && getenv("SPAND_QC_VEC")) ? atoi(getenv("SPAND_QC_VEC")) : -1;
        // SPAND_QC_CS=<cs>, SPAND_QC_THREADS=<n>: that configuration wherever the matrices
        // fit (measurement aids)
        const int force = (honour_force && getenv("SPAND_QC_CS")) ? atoi(getenv("SPAND_QC_CS")) : 0;
        const int force_th = (honour_force && getenv("SPAND_QC_THREADS")) ? atoi(getenv("SPAND_QC_THREADS")) : 0;
        for (int cs = 1; cs <= qc_max_cs_; cs *= 2) {
            int64_t sm = 4096, work = 0;
            for (const auto& d : dims) {
                sm = std::max<int64_t>(sm, qc_need(d.first, d.second, cs, (int)sizeof(T)));
                work = std::max(work, (int64_t)d.first * ((d.second + cs - 1) / cs));
            }
            sm = (sm + 255) & ~int64_t(255);
            if (sm > qc_smem_cap_) continue;
            for (int th = 64; th <= QC_WIDE_THREADS; th *= 2) {
                if (th > QC_THREADS && sm > qcw_smem_cap_) continue;
                const int active = active_clusters(W.n * cs, cs, (int)sm, th, qrcp_smem_kernel_ptr<T>(th));
                if (active <= 0) continue;
                const int rounds = (W.n + active - 1) / active;
                // per pivot step: barrier latency + the passes over the largest slab (the
                // kernel is latency-bound: CTAs sharing an SM do not slow each other down much)
                double est = rounds * (3000.0 + 500.0 * std::log2((double)cs) +
                                       5.0 / 32.0 * (double)work * ((double)QC_THREADS / th));
                if (force > 0 && cs != force) est = 1e200;
                if (force_th > 0 && th != force_th) est = 1e200;
                // the same launch with the vectorised update for slabs of QC_VEC_FROM rows or
                // more (faster on the 200-400-row matrices of the top levels, slower below)
                const bool vec_ok = maxrows_ >= QC_VEC_FROM && force_vec != 0;
                const double est_vec = (vec_ok && est < 1e200) ? est * (maxrows_ >= 2 * QC_VEC_FROM ? 0.9 : 1.1) : 1e200;
                const bool take_vec = force_vec == 1 ? vec_ok : (vec_ok && est_vec < est);
                if (est < 1e200) all.push_back(QcConf{0, cs, th, (int)sm, INT_MAX, est});
                if (est_vec < 1e200) all.push_back(QcConf{0, cs, th, (int)sm, QC_VEC_FROM, est_vec});
                const double e = take_vec ? est_vec : est;
                if (e < best) {
                    best = e;
                    bcs = cs;
                    bsm = (int)sm;
                    bth = th;
                    bvec = take_vec ? QC_VEC_FROM : INT_MAX;
                }
            }
        }
        // the blocked kernel (plain QRCP only): one read of the slab per pivot step and a
        // panel update every QB_NB steps instead of four loads and a store per element.
        // Measured on GB300 it is slower than the unblocked kernel at every wave (the step
        // is bound by latency, not by shared-memory bandwidth), so it is taken only with
        // SPAND_QC_BLOCKED=1 (wherever the matrices fit it)
        int brpl = 0;
        const char* fb = honour_force ? getenv("SPAND_QC_BLOCKED") : nullptr;
        const int force_b = fb ? atoi(fb) : 0;
        int maxrows = 0;
        for (const auto& d : dims) maxrows = std::max(maxrows, d.first);
        const int rpl = qb_rpl(maxrows);
        if (rpl > 0 && !(nphi_ && pres_adaptive_) && force_b != 0) {
            const QcKernel<T> fn = qrcp_blocked_kernel_ptr<T>(rpl);
            if (force_b == 1) best = 1e300;
            for (int cs = 1; cs <= qc_max_cs_; cs *= 2) {
                int64_t sm = 4096, work = 0;
                for (const auto& d : dims) {
                    sm = std::max<int64_t>(sm, qb_need(d.first, d.second, cs, (int)sizeof(T)));
                    work = std::max(work, (int64_t)d.first * ((d.second + cs - 1) / cs));
                }
                sm = (sm + 255) & ~int64_t(255);
                if (sm > qb_smem_cap_) continue;
                for (int th = 64; th <= QC_THREADS; th *= 2) {
                    const int active = active_clusters(W.n * cs, cs, (int)sm, th, fn);
                    if (active <= 0) continue;
                    const int rounds = (W.n + active - 1) / active;
                    double est = rounds * (4500.0 + 500.0 * std::log2((double)cs) +
                                           1.5 / 32.0 * (double)work * ((double)QC_THREADS / th));
                    if (force > 0 && cs != force) est = 1e200;
                    if (force_th > 0 && th != force_th) est = 1e200;
                    if (est < 1e200) all.push_back(QcConf{rpl, cs, th, (int)sm, INT_MAX, est});
                    if (est < best) {
                        best = est;
                        bcs = cs;
                        bsm = (int)sm;
                        bth = th;
                        brpl = rpl;
                        bvec = INT_MAX;
                    }
                }
            }
        }
        W.gskip = false;
        if (!bcs) {  // matrices above the cap take the global-memory path
            W.rpl = 0;
            W.vec_rows = INT_MAX;
            W.cs = qc_max_cs_;
            W.smem = qc_smem_cap_;
            W.threads = QC_THREADS;
            return;
        }
        W.rpl = brpl;
        W.vec_rows = bvec;
        W.cs = bcs;
        W.smem = bsm;
        W.threads = bth;
        W.cands.clear();
        W.timed.clear();
        // every candidate holds the matrices at these sizes: the global pass is not queued
        W.gskip = gskip_on_ && !force_global_;
        if (collect && force_b == 0 && force <= 0 && force_th <= 0 && force_vec < 0) {
            // the measuring factorization times the model's best configurations of each
            // kernel variant (QC_TUNE_PER_KIND each: scalar, blocked, vectorised update; the
            // model's pick first)
            std::stable_sort(all.begin(), all.end(), [](const QcConf& a, const QcConf& b) { return a.est < b.est; });
            W.cands.push_back(QcConf{brpl, bcs, bth, bsm, bvec, best});
            int taken[3] = {0, 0, 0};
            for (const QcConf& q : all) {
                const int kind = q.rpl > 0 ? 1 : (q.vec_rows < INT_MAX ? 2 : 0);
                if (taken[kind] >= QC_TUNE_PER_KIND) continue;
                taken[kind]++;
                if (q.rpl == brpl && q.cs == bcs && q.threads == bth && q.vec_rows == bvec) continue;
                W.cands.push_back(q);
            }
            // and the model pick's neighbours (twice the CTAs with half or the same threads,
            // half the CTAs with twice the threads, half the threads): where the model errs
            // the fastest launch was one of these at 64^3
            const int nb[4][2] = {{2, -2}, {2, 1}, {-2, 2}, {1, -2}};
            for (const auto& m : nb) {
                const int cs = m[0] > 0 ? bcs * m[0] : bcs / -m[0];
                const int th = m[1] > 0 ? bth * m[1] : bth / -m[1];
                for (const QcConf& q : all) {
                    if (q.rpl || q.cs != cs || q.threads != th || q.vec_rows != bvec) continue;
                    bool dup = false;
                    for (const QcConf& c : W.cands)
                        dup |= c.rpl == q.rpl && c.cs == q.cs && c.threads == q.threads && c.vec_rows == q.vec_rows;
                    if (!dup) W.cands.push_back(q);
                }
            }
        }
    }
    static constexpr int QC_VEC_FROM = 128;  // the vectorised update's candidates: slabs of >= 128 rows
    static constexpr int QC_TUNE_PER_KIND = 3;
    QcProj<T> qc_proj() const {
        if (nphi_ && pres_adaptive_) return QcProj<T>{vstore_, rank1_};
        return QcProj<T>{nullptr, nullptr};
    }
    PhiCtx<T> phictx() const { return PhiCtx<T>{phis_, d_phioff_, nphi_}; }
    void launch_qrcp_global(WaveDev& W, double tol) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)(W.n * W.gcs));
        cfg.blockDim = dim3(QC_THREADS);
        cfg.dynamicSmemBytes = (size_t)W.gsmem;
        cfg.stream = s_;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)W.gcs;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        SPAND_CUDA(cudaLaunchKernelEx(&cfg, qrcp_gslab_kernel_ptr<T>(), ctx_, (const DSpars*)W.items,
                                      (const DAsn*)pieces_, ws_, ws2_, jpvt_, ipvt_, tauws_, rank_, colcount_,
                                      fallback_, tol, W.gsmem, INT_MAX, qc_proj()));
    }
    void apply_conf(WaveDev& W, const QcConf& q) {
        W.vec_rows = q.vec_rows;
        W.rpl = q.rpl;
        W.cs = q.cs;
        W.threads = q.threads;
        W.smem = q.smem;
        W.cands.clear();
    }
    std::vector<QrcpWave> qrcp_waves() const override {
        std::vector<QrcpWave> out;
        for (size_t l = 0; l < levels_.size(); l++)
            for (size_t w = 0; w < levels_[l].waves.size(); w++) {
                const WaveDev& W = levels_[l].waves[w];
                QrcpWave q;
                const int c[9] = {(int)l, (int)w, W.n, W.maxcap, W.rpl, W.cs, W.threads, W.smem, W.vec_rows};
                std::copy(c, c + 9, q.conf);
                for (const auto& t : W.timed) {
                    q.cand.push_back({t.first.rpl, t.first.cs, t.first.threads, t.first.smem, t.first.vec_rows});
                    q.ms.push_back(t.second);
                }
                out.push_back(q);
            }
        return out;
    }
    size_t n_waves() const {
        size_t n = 0;
        for (const LevelDev& D : levels_) n += D.waves.size();
        return n;
    }
    // Measured choice: every candidate of the wave on the same inputs (the kernel only
    // reads the edge blocks and sizes and rewrites its own outputs), timed with events on
    // the stream, then the fastest once more so that its outputs are the ones that stay.
    void launch_qrcp_cluster(WaveDev& W, double tol) {
        if (!measuring_ || W.cands.size() < 2) {
            launch_qrcp_once(W, tol);
            return;
        }
        const size_t K = W.cands.size();
        while (tune_ev_.size() < 2 * K) {
            cudaEvent_t e;
            SPAND_CUDA(cudaEventCreate(&e));
            tune_ev_.push_back(e);
        }
        // one untimed launch first, so that every timed one finds the inputs in L2 alike;
        // every candidate timed twice (rounds in the same order), the faster kept
        apply_conf_keep(W, W.cands[0]);
        launch_qrcp_once(W, tol);
        std::vector<float> best_ms(K, 1e30f);
        for (int round = 0; round < 2; round++) {
            for (size_t k = 0; k < K; k++) {
                apply_conf_keep(W, W.cands[k]);
                SPAND_CUDA(cudaEventRecord(tune_ev_[2 * k], s_));
                launch_qrcp_once(W, tol);
                SPAND_CUDA(cudaEventRecord(tune_ev_[2 * k + 1], s_));
            }
            SPAND_CUDA(cudaEventSynchronize(tune_ev_[2 * K - 1]));
            for (size_t k = 0; k < K; k++) {
                float ms = 0;
                SPAND_CUDA(cudaEventElapsedTime(&ms, tune_ev_[2 * k], tune_ev_[2 * k + 1]));
                best_ms[k] = std::min(best_ms[k], ms);
            }
        }
        size_t bk = 0;
        float bms = 1e30f;
        W.timed.clear();
        for (size_t k = 0; k < K; k++) {
            const float ms = best_ms[k];
            W.timed.push_back({W.cands[k], ms});
            if (ms < bms) {
                bms = ms;
                bk = k;
            }
        }
        const QcConf q = W.cands[bk];
        apply_conf(W, q);
        launch_qrcp_once(W, tol);
        launches_ += (int64_t)(2 * K + 1);
    }
    void apply_conf_keep(WaveDev& W, const QcConf& q) {
        W.vec_rows = q.vec_rows;
        W.rpl = q.rpl;
        W.cs = q.cs;
        W.threads = q.threads;
        W.smem = q.smem;
    }
    void launch_qrcp_once(WaveDev& W, double tol) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)(W.n * W.cs));
        cfg.blockDim = dim3((unsigned)W.threads);
        cfg.dynamicSmemBytes = force_global_ ? 0 : (size_t)W.smem;
        cfg.stream = s_;
        cudaLaunchAttribute attr[2];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)W.cs;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        // a programmatic dependent of the previous launch (as launch_pdl) when the blocked
        // kernel, whose body does not wait, is not the one launched
        if (pdl_on_ && !prof_.enabled() && !check_launches_ && !measuring_ && !(W.rpl > 0 && !force_global_)) {
            attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
            attr[1].val.programmaticStreamSerializationAllowed = 1;
            cfg.numAttrs = 2;
        }
        const QcKernel<T> fn =
            W.rpl > 0 && !force_global_ ? qrcp_blocked_kernel_ptr<T>(W.rpl) : qrcp_smem_kernel_ptr<T>(W.threads);
        SPAND_CUDA(cudaLaunchKernelEx(&cfg, fn, ctx_, (const DSpars*)W.items, (const DAsn*)pieces_, ws_, (T*)nullptr,
                                      jpvt_, ipvt_, tauws_, rank_, colcount_, fallback_, tol,
                                      force_global_ ? 0 : W.smem, W.vec_rows, qc_proj()));
    }
    void launch_potrf(int* pivots, int* clusters, int n, const int* ps_piv, const int* ps_cl, int n_ps,
                      const int* pb_piv, const int* pb_cl, int n_pb, int smem, const TrtriDev& tri, int pc_cs,
                      int pc_smem, bool split_pays) {
        // (not beside the cluster kernel or the strip inverse, which take every pivot of the list)
        const bool small = n_ps > 0 && potrf_small_on_ && pc_cs == 0 && smem > 0;
        if (small)
            launch("potrf", [&] {
                launch_pdl(potrf_small_kernel<T>, dim3((n_ps + PS_WARPS - 1) / PS_WARPS), dim3(32 * PS_WARPS), 0, 1,
                           ctx_, ps_piv, ps_cl, n_ps);
            });
        if (pc_cs > 0) {
            launch("potrf_cluster", [&] {
                launch_pdl(potrf_cluster_kernel<T>, dim3((unsigned)(n * pc_cs)), dim3(PC_THREADS), (size_t)pc_smem,
                           pc_cs, ctx_, (const int*)pivots, (const int*)clusters, n, pc_smem, pc_fallback_);
            });
        }
        // The strip-wise inverse runs only where pivots may miss the single-CTA kernel's shared
        // memory (which inverts what it holds); without it potrf3 inverts every pivot itself.
        const bool strips = tri.ntiles > 0 && (smem == 0 || pc_cs > 0);
        // single-CTA kernel: every pivot, or (after the cluster kernel) those it could not hold,
        // or (beside the warp kernel) the pivots of more than 32 rows only
        // Where a few large pivots set the level's shared memory (potrf_split_pays), the pivots
        // of at most mid_n rows run first in a launch sized for them, more CTAs per SM, then
        // the larger ones (each launch skips the other class's pivots at once).
        const int mid_n = potrf_mid_n();
        const bool split = split_pays && potrf_split_on_ && pc_cs == 0 && smem > POTRF_MID_SMEM;
        const int mid_smem = (int)(potrf_held(mid_n) * (int64_t)sizeof(T));
        const int tiled = potrf_tiled_on_ ? 1 : 0;
        if (small && n_pb == 0) {
        } else if (small) {
            if (split)
                launch("potrf", [&] {
                    launch_pdl(potrf3_kernel<T>, dim3(n_pb), dim3(256), (size_t)mid_smem, 1, ctx_, pb_piv, pb_cl, n_pb,
                               mid_smem / (int)sizeof(T), 0, (const int*)nullptr, 0, tiled, 0, mid_n);
                });
            launch("potrf", [&] {
                launch_pdl(potrf3_kernel<T>, dim3(n_pb), dim3(256), (size_t)smem, 1, ctx_, pb_piv, pb_cl, n_pb,
                           smem / (int)sizeof(T), 0, (const int*)nullptr, 0, tiled, split ? mid_n : 0, INT_MAX);
            });
        } else {
            const int strip_max_n = strips ? tri.smem / (32 * (int)sizeof(T)) : 0;
            if (split)
                launch("potrf", [&] {
                    launch_pdl(potrf3_kernel<T>, dim3(n), dim3(256), (size_t)mid_smem, 1, ctx_, (const int*)pivots,
                               (const int*)clusters, n, mid_smem / (int)sizeof(T), strip_max_n, (const int*)nullptr, 0,
                               tiled, 0, mid_n);
                });
            launch("potrf", [&] {
                launch_pdl(potrf3_kernel<T>, dim3(n), dim3(256), (size_t)smem, 1, ctx_, (const int*)pivots,
                           (const int*)clusters, n, smem / (int)sizeof(T), strip_max_n,
                           pc_cs > 0 ? (const int*)pc_fallback_ : nullptr, 0, tiled, split ? mid_n : 0, INT_MAX);
            });
        }
        if (strips)
            launch("trtri", [&] {
                launch_pdl(trtri_kernel<T>, dim3(tri.ntiles), dim3(256), (size_t)tri.smem, 1, ctx_, (const int*)pivots,
                           (const int*)clusters, (const DTile*)tri.tiles, tri.ntiles, tri.smem / (int)sizeof(T),
                           pc_cs > 0 ? 0LL : (long long)(smem / (int)sizeof(T)));
            });
    }
    void launch_getrf(int* pivots, int* invs, int* clusters, int n, int smem) {
        launch("getrf", [&] {
            getrf_kernel<T><<<n, LU_THREADS, smem, s_>>>(ctx_, pivots, invs, clusters, n, smem / (int)sizeof(T),
                                                          lu_perm_, lu_swp_, d_xoff_);
        });
    }
    void launch_ldlt(int* pivots, int* clusters, int* newpiv, int n, int smem) {
        if (!n) return;
        launch("ldlt", [&] {
            ldlt_kernel<T><<<n, LU_THREADS, smem, s_>>>(ctx_, pivots, clusters, newpiv, n, smem / (int)sizeof(T),
                                                         lu_perm_, lu_swp_, signs_, d_xoff_);
        });
    }
    static int lu_smem_n(int64_t mx) {
        const int64_t full = (mx * mx + mx) * (int64_t)sizeof(T);
        if (full <= 200 * 1024) return (int)full;
        return (int)(mx * sizeof(T));
    }
    void launch_lu_trsm(const TrsmDev& t) {
        if (!t.ntiles) return;
        launch("trsm", [&] {
            lu_trsm_kernel<T><<<t.ntiles, 256, t.smem, s_>>>(ctx_, t.items, t.tiles, t.ntiles, t.smem / (int)sizeof(T),
                                                             lu_perm_, lu_swp_, d_xoff_);
        });
    }
    // shared memory of the PLU pivot kernel: the whole block and one column where it fits,
    // else the column alone (the block is then worked on in global memory)
    int lu_smem_for(const std::vector<int>& clusters, const Plan& P) {
        int64_t mx = 1;
        for (int c0 : clusters) mx = std::max<int64_t>(mx, P.c_cap[c0]);
        const int64_t full = (mx * mx + mx) * (int64_t)sizeof(T);
        if (full <= 200 * 1024) return (int)full;
        if (mx * (int64_t)sizeof(T) > 200 * 1024) throw DeviceError{SPAND_ERR_UNSUPPORTED, "pivot too large"};
        return (int)(mx * sizeof(T));
    }
    // A kernel of the factorization's main stream or of the one-right-hand-side solve sweep,
    // launched as a programmatic dependent of the previous one (its CTAs are scheduled while
    // that one still runs and wait in pdl_wait_and_release for its completion): chains of
    // hundreds of dependent launches overlap their launch latency.  Off while the profiler
    // or the measuring factorization times launches one by one, and with SPAND_PDL=0.
    template <typename... KArgs, typename... Args>
    void launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, int cluster, Args&&... args) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = grid;
        cfg.blockDim = block;
        cfg.dynamicSmemBytes = smem;
        cfg.stream = s_;
        cudaLaunchAttribute attr[2];
        int na = 0;
        if (cluster > 1) {
            attr[na].id = cudaLaunchAttributeClusterDimension;
            attr[na].val.clusterDim.x = (unsigned)cluster;
            attr[na].val.clusterDim.y = 1;
            attr[na].val.clusterDim.z = 1;
            na++;
        }
        if (pdl_on_ && !prof_.enabled() && !check_launches_ && !measuring_) {
            attr[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
            attr[na].val.programmaticStreamSerializationAllowed = 1;
            na++;
        }
        cfg.attrs = attr;
        cfg.numAttrs = na;
        SPAND_CUDA(cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...));
    }
    void launch_schur(const DTarget* targets, const DUpd* ups, const DTile* tiles, int ntiles) {
        if (!ntiles) return;
        if constexpr (sizeof(T) == 4) {
            if (schur_tc_on_) {
                launch("schur", [&] {
                    launch_pdl(schur_tc_kernel, dim3(ntiles), dim3(256), 0, 1, ctx_, targets, ups, tiles, ntiles,
                               (const float*)signs_, (const long long*)d_xoff_);
                });
                return;
            }
        }
        launch("schur", [&] {
            launch_pdl(schur_kernel<T>, dim3(ntiles), dim3(256), 0, 1, ctx_, targets, ups, tiles, ntiles,
                       (const T*)signs_, (const long long*)d_xoff_);
        });
    }
    void launch_trsm(const TrsmDev& t) {
        if (!t.ntiles) return;
        if constexpr (sizeof(T) == 4) {
            // FP32 path, LLT pivots: the tensor-core kernel wherever its staged tile fits
            const int nmax = t.smem / (TRB * (int)sizeof(T));
            const int64_t tcs = (int64_t)TC_XLD * ((nmax + 7) & ~7) * (int64_t)sizeof(float);
            if (trsm_tc_on_ && !ldlt_ && t.smem > 16 && tcs <= 200 * 1024) {
                // pivots of at most 32 rows a warp per tile, the others a CTA per tile
                const bool split = trsm_small_on_ && t.nstiles > 0;
                if (split)
                    launch("trsm", [&] {
                        launch_pdl(trsm_tc_small_kernel, dim3((t.nstiles + TSW - 1) / TSW), dim3(32 * TSW), 0, 1, ctx_,
                                   (const DTrsm*)t.items, (const DTile*)t.stiles, t.nstiles);
                    });
                const int nb = split ? t.nbtiles : t.ntiles;
                if (nb)
                    launch("trsm", [&] {
                        launch_pdl(trsm_tc_kernel, dim3(nb), dim3(256), (size_t)tcs, 1, ctx_, (const DTrsm*)t.items,
                                   (const DTile*)(split ? t.btiles : t.tiles), nb);
                    });
                return;
            }
        }
        launch("trsm", [&] {
            launch_pdl(trsm3_kernel<T>, dim3(t.ntiles), dim3(256), (size_t)t.smem, 1, ctx_, (const DTrsm*)t.items,
                       (const DTile*)t.tiles, t.ntiles, t.smem / (int)sizeof(T),
                       (const int*)(ldlt_ ? lu_perm_ : nullptr), (const long long*)d_xoff_);
        });
    }
    // Cluster Cholesky for pivots of up to nmax rows that one CTA's shared memory cannot
    // hold (cs = 0: keep the single-CTA kernel).  The panels' trailing updates are spread
    // over the cluster, so a larger cluster shortens each panel step: among the clusters
    // whose CTAs hold their panels, the largest with at least one panel per CTA whose
    // CTAs all fit on the GPU at once (else the smallest that fits).
    void choose_potrf_cluster(int nmax, int single_smem, int count, int& cs_out, int& smem_out) {
        cs_out = 0;
        smem_out = 0;
        if (single_smem > 0 || count == 0) return;
        const int np = (nmax + 31) / 32;
        for (int cs = 2; cs <= qc_max_cs_; cs *= 2) {
            const long long need = (pc_need(nmax, cs, 0, (int)sizeof(T)) + 255) & ~255LL;
            if (need > pc_smem_cap_) continue;
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3((unsigned)(count * cs));
            cfg.blockDim = dim3(PC_THREADS);
            cfg.dynamicSmemBytes = (size_t)need;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = (unsigned)cs;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            int active = 0;
            if (cudaOccupancyMaxActiveClusters(&active, potrf_cluster_kernel<T>, &cfg) != cudaSuccess) {
                cudaGetLastError();
                continue;
            }
            if (active <= 0) continue;
            const bool first = cs_out == 0;
            if (first || (active >= count && cs <= np)) {
                cs_out = cs;
                smem_out = (int)need;
            }
            if (!first && (active < count || cs > np)) break;
        }
    }
    // shared memory of the POTRF kernel for pivots of size up to nmax: whole block, else one panel
    // CTAs of the one-CTA Cholesky per SM at `smem` bytes of dynamic shared memory (its
    // register bound: three in FP32, two in FP64)
    int potrf_ctas_per_sm(int smem) const {
        const int per = smem + PNB * (PNB + 1) * (int)sizeof(T) + 1024;
        return std::max(1, std::min(sizeof(T) == 4 ? 3 : 2, (228 * 1024) / per));
    }
    // Size classes pay where at most eight pivots (by their sizes in the first factorization)
    // exceed mid_n rows and the others would take fewer waves of CTAs at the smaller launch's
    // occupancy; otherwise the second launch only adds its length (measured at 64^3: the
    // lowest level's elimination 0.35 -> 0.27 ms; levels with tens of large pivots slower).
    bool potrf_split_pays(const std::vector<int>& cl, const std::vector<int>& r0, int smem) const {
        const int mid_n = potrf_mid_n();
        int big = 0, mid = 0;
        for (int c0 : cl) {
            if (P_->c_cap[c0] <= 32) continue;  // the warp kernel's
            if (r0[c0] > mid_n) big++;
            else mid++;
        }
        if (big > 8 || smem <= POTRF_MID_SMEM) return false;
        const long long full = (long long)num_sms_ * potrf_ctas_per_sm(smem);
        const long long part = (long long)num_sms_ * potrf_ctas_per_sm((int)(potrf_held(mid_n) * (int64_t)sizeof(T)));
        return (mid + full - 1) / full > (mid + part - 1) / part;
    }
    // largest pivot the size-class launch of the one-CTA Cholesky holds in POTRF_MID_SMEM
    static int potrf_mid_n() {
        int m = 32;
        while (potrf_held(m + 1) * (int64_t)sizeof(T) <= POTRF_MID_SMEM) m++;
        return m;
    }
    static int potrf_smem_n(int nmax) {
        int64_t full = potrf_held(nmax) * (int64_t)sizeof(T);
        return full <= POTRF_SMEM_MAX ? (int)std::max<int64_t>(full, 16) : 0;
    }
    // the strip (32 columns) and, where it fits, the staged row-block tile (33 columns)
    static int trtri_smem_n(int nmax) {
        const int64_t b = (int64_t)65 * nmax * sizeof(T);
        if (b <= 200 * 1024) return (int)std::max<int64_t>(b, 16);
        return (int)std::min<int64_t>((int64_t)32 * nmax * sizeof(T), 200 * 1024);
    }
    TrtriDev build_trtri(const std::vector<int>& clusters, const Plan& P) {
        std::vector<int> ext;
        int mx = 0;
        for (int c0 : clusters) {
            ext.push_back(P.c_cap[c0]);
            mx = std::max(mx, P.c_cap[c0]);
        }
        auto t = tiles_1d(ext, 32);
        return {up(t), (int)t.size(), trtri_smem_n(mx)};
    }
    static int trsm_smem_n(int nmax) {
        int64_t b = (int64_t)TRB * nmax * sizeof(T);
        return b <= 200 * 1024 ? (int)std::max<int64_t>(b, 16) : 0;
    }
    int trsm_smem(const std::vector<int>& clusters, const Plan& P) {
        int mx = 0;
        for (int c0 : clusters) mx = std::max(mx, P.c_cap[c0]);
        return trsm_smem_n(mx);
    }

    void run_solve(double* x, int nrhs, int ld) { run_solve_slots(x, nrhs, ld, xs_, xs_ + (size_t)xld_ * x_nrhs_); }

    // the Cholesky-layout triangular products on a list of LDLT pivots (siblings)
    void trsv_ldlt(const int* clusters, const int* blks, const int2* tv, int ntv, int smem, int trans, XCtx<T> X,
                   T* tmp) {
        if (!ntv) return;
        launch("trsv", [&] {
            trsv4_kernel<T><<<ntv, TV_THREADS, smem, s_>>>(ctx_, X, clusters, blks, tv, trans, tmp, tv_count_);
        });
    }

    // slots: the solve vectors (xld x nrhs); tmp: their scratch copy, same layout
    void run_solve_slots(double* x, int nrhs, int ld, T* slots, T* tmp) {
        const Plan& P = *P_;
        XCtx<T> X{slots, (long long)xld_, d_xoff_, nrhs};
        const int n = (int)perm_h_.size();
        const long long tot = (long long)n * nrhs;
        // 16 or more right-hand sides: the kernels that read each factor block once per 32
        // (not on the LDLT path, whose sweeps carry signs and permutations)
        const bool mr = nrhs >= 16 && !ldlt_ && !lorasp_;
        const T* sg = ldlt_ ? signs_ : nullptr;
        auto permx = [&](const int* clusters, int count, int fwd, int smem) {
            if (!ldlt_ || !count) return;
            launch("perm_x", [&] {
                perm_x_kernel<T><<<dim3((unsigned)count, (unsigned)nrhs), 256, smem, s_>>>(ctx_, X, clusters, count,
                                                                                         lu_perm_, d_xoff_, fwd);
            });
        };
        auto siblings = [&](LevelDev& D, int fwd) {
            if (!(ldlt_ || lorasp_) || !D.n_sib) return;
            auto split = [&] {
                launch("split_x", [&] {
                    split_x_kernel<T><<<dim3((unsigned)D.n_sib, (unsigned)nrhs), 128, 0, s_>>>(
                        ctx_, X, D.sib_owner, D.sib_clusters, D.n_sib, fwd);
                });
            };
            if (fwd) {
                split();
                if (ldlt_) {  // LoRaSp siblings have the identity for pivot
                    permx(D.sib_clusters, D.n_sib, 1, D.x_smem_sib);
                    trsv_ldlt(D.sib_clusters, D.sib_piv, D.sib_tv, D.n_sib_tv, D.x_smem_sib, 0, X, tmp);
                }
                if (D.n_sib_gf_tiles)
                    launch("gemm_fwd", [&] {
                        gemm_fwd2_kernel<T><<<D.n_sib_gf_tiles * nrhs, 256, 0, s_>>>(
                            ctx_, X, D.sib_gf, D.sib_gfo, D.sib_gf_tiles, D.n_sib_gf_tiles, 0, signs_, d_xoff_,
                            ldlt_ ? 1 : 0);
                    });
            } else {
                if (D.n_sib_gb_tiles)
                    launch("gemm_bwd", [&] {
                        gemm_bwd2_kernel<T><<<D.n_sib_gb_tiles * nrhs, 256, 0, s_>>>(
                            ctx_, X, D.sib_gb, D.sib_gbo, D.sib_gb_tiles, D.n_sib_gb_tiles, signs_, d_xoff_,
                            ldlt_ ? 1 : 0);
                    });
                if (ldlt_) {
                    trsv_ldlt(D.sib_clusters, D.sib_piv, D.sib_tv, D.n_sib_tv, D.x_smem_sib, 1, X, tmp);
                    permx(D.sib_clusters, D.n_sib, 0, D.x_smem_sib);
                }
                split();
            }
        };
        launch("perm", [&] {
            launch_pdl(perm_in_kernel<T>, dim3((unsigned)((tot + 255) / 256)), dim3(256), 0, 1, (const double*)x, ld, X,
                         (const int*)d_perm_, (const long long*)d_slot_, n);
        });
        auto trsv_mr = [&](const int* clusters, const int* blks, const int* small, int nsmall, const int2* big, int nbig,
                           int trans) {
            const int nrbk = (nrhs + MR_RB - 1) / MR_RB;
            if (nsmall)
                launch("trsv", [&] {
                    const unsigned g = (unsigned)((nsmall * nrbk + MRS_WARPS - 1) / MRS_WARPS);
                    trsv_mrhs_small_kernel<T><<<g, 32 * MRS_WARPS, MRS_WARPS * MR_MAXROWS * (MR_RB + 1) * sizeof(T), s_>>>(
                        ctx_, X, clusters, blks, small, nsmall, trans);
                });
            if (nbig)
                launch("trsv", [&] {
                    trsv_mrhs_kernel<T><<<nbig, 256, 0, s_>>>(ctx_, X, clusters, blks, big, trans, tmp, tv_count_);
                });
        };
        auto trsv = [&](const int* clusters, const int* blks, const int2* tv, int ntv, int smem, int trans) {
            if (!ntv) return;
            if (mr && !lu_) {
                const LevelDev& D = levels_[cur_level_];
                if (clusters == D.elim_llt)
                    trsv_mr(clusters, blks, D.elim_small, D.n_elim_small, D.elim_big_tv, D.n_elim_big_tv, trans);
                else
                    trsv_mr(clusters, blks, D.scale_small, D.n_scale_small, D.scale_big_tv, D.n_scale_big_tv, trans);
                return;
            }
            if (lu_) {
                // PLU: blks are the inverse blocks; one CTA per (cluster, right-hand side)
                const int count = cur_count_;
                launch("trsv", [&] {
                    lu_apply_kernel<T><<<dim3((unsigned)count, (unsigned)nrhs), 256, smem, s_>>>(
                        ctx_, X, clusters, blks, count, lu_perm_, d_xoff_, trans ? 0 : 1);
                });
                return;
            }
            if (!mr && trsv_small_on_ && cur_level_ >= 0) {
                // clusters of at most 64 rows a warp each, the others in row tiles
                const LevelDev& D = levels_[cur_level_];
                const bool elim = clusters == D.elim_llt;
                const bool scale = clusters == D.scale_llt;
                if (elim || scale) {
                    const int* small = elim ? D.elim_small : D.scale_small;
                    const int nsmall = elim ? D.n_elim_small : D.n_scale_small;
                    const int2* big = elim ? D.elim_big_tv : D.scale_big_tv;
                    const int nbig = elim ? D.n_elim_big_tv : D.n_scale_big_tv;
                    const int nsb = (nsmall + TS_WARPS - 1) / TS_WARPS;
                    if (nsmall && nbig && trsv_fuse_on_) {
                        launch("trsv", [&] {
                            launch_pdl(trsv_fused_kernel<T>, dim3((unsigned)(nsb + nbig)), dim3(TV_THREADS),
                                         (size_t)smem, 1, ctx_, X, clusters, blks, small, nsmall, nsb, big, trans, tmp,
                                         tv_count_);
                        });
                        return;
                    }
                    if (nsmall)
                        launch("trsv", [&] {
                            launch_pdl(trsv_small_kernel<T>, dim3(nsb), dim3(32 * TS_WARPS), 0, 1, ctx_, X, clusters,
                                         blks, small, nsmall, trans);
                        });
                    if (nbig)
                        launch("trsv", [&] {
                            launch_pdl(trsv4_kernel<T>, dim3(nbig), dim3(TV_THREADS), (size_t)smem, 1, ctx_, X,
                                         clusters, blks, big, trans, tmp, tv_count_);
                        });
                    return;
                }
            }
            launch("trsv", [&] {
                if (mr)
                    trsv_mrhs_kernel<T><<<ntv, 256, 0, s_>>>(ctx_, X, clusters, blks, tv, trans, tmp, tv_count_);
                else
                    launch_pdl(trsv4_kernel<T>, dim3(ntv), dim3(TV_THREADS), (size_t)smem, 1, ctx_, X, clusters, blks,
                                 tv, trans, tmp, tv_count_);
            });
        };
        auto ortho = [&](const LevelDev& D, int trans) {
            if (!D.n_ortho) return;
            launch("ortho", [&] {
                if (mr && D.ortho_mrhs_smem)
                    ortho_mrhs_kernel<T><<<D.n_ortho, 256, D.ortho_mrhs_smem, s_>>>(ctx_, X, D.ortho, vstore_, tstore_,
                                                                                    trans);
                else if (D.ortho_cs > 1 && ortho_full_on_ && ortho_cluster_on_)
                    launch_pdl(ortho_cluster_kernel<T, 256>, dim3((unsigned)(D.n_ortho * nrhs * D.ortho_cs)), dim3(256),
                                 (size_t)D.ortho_cs_smem, D.ortho_cs, ctx_, X, (const DOrtho*)D.ortho, D.n_ortho,
                                 (const T*)vstore_, (const T*)tstore_, trans);
                else if (D.ortho_full_smem && ortho_full_on_) {
                    if (D.ortho_full_wide)
                        launch_pdl(ortho_full_kernel<T, 512>, dim3(D.n_ortho * nrhs), dim3(512),
                                     (size_t)D.ortho_full_smem, 1, ctx_, X, (const DOrtho*)D.ortho, D.n_ortho,
                                     (const T*)vstore_, (const T*)tstore_, trans);
                    else
                        launch_pdl(ortho_full_kernel<T, 256>, dim3(D.n_ortho * nrhs), dim3(256),
                                     (size_t)D.ortho_full_smem, 1, ctx_, X, (const DOrtho*)D.ortho, D.n_ortho,
                                     (const T*)vstore_, (const T*)tstore_, trans);
                } else
                    launch_pdl(ortho_wyb_kernel<T>, dim3(D.n_ortho * nrhs), dim3(512), (size_t)D.x_smem_ortho, 1,
                                 ctx_, X, (const DOrtho*)D.ortho, D.n_ortho, (const T*)vstore_, (const T*)tstore_,
                                 trans, D.x_smem_ortho / (int)sizeof(T));
            });
        };
        auto merge = [&](const LevelDev& D, int fwd) {
            if (!(D.merged && D.n_children)) return;
            launch("merge_x", [&] {
                if (mr)
                    merge_x_mrhs_kernel<T><<<D.n_children, 256, 0, s_>>>(ctx_, X, D.child_idx, D.child_parent, cpos_, fwd);
                else
                    launch_pdl(merge_x_kernel<T>, dim3((D.n_children * nrhs + 7) / 8), dim3(256), 0, 1, ctx_, X,
                                 (const int*)D.child_idx, (const int*)D.child_parent, D.n_children,
                                 (const int*)cpos_, fwd);
            });
        };
        for (int l = 0; l < P.nlevels; l++) {
            LevelDev& D = levels_[l];
            cur_level_ = l;
            cur_count_ = D.n_elim_llt;
            permx(D.elim_llt, D.n_elim_llt, 1, D.x_smem_elim);
            trsv(D.elim_llt, lu_ ? D.elim_inv : D.elim_llt_blk, D.elim_tv, D.n_elim_tv, D.x_smem_elim, 0);
            if (D.n_gf && D.n_gf_tiles)
                launch("gemm_fwd", [&] {
                    if (mr)
                        gemm_mrhs_kernel<T><<<D.n_gf_tiles32, 256, 0, s_>>>(ctx_, X, D.gf, D.gfo, D.gf_tiles32, 1);
                    else
                        launch_pdl(gemm_fwd2_kernel<T>, dim3(D.n_gf_tiles * nrhs), dim3(256), 0, 1, ctx_, X,
                                     (const DGroup*)D.gf, (const DGemmOp*)D.gfo, (const DTile*)D.gf_tiles,
                                     D.n_gf_tiles, 0, sg, (const long long*)d_xoff_, 0);
                });
            cur_count_ = D.n_scale_llt;
            permx(D.scale_llt, D.n_scale_llt, 1, D.x_smem_scale);
            trsv(D.scale_llt, lu_ ? D.scale_inv : D.scale_llt_blk, D.scale_tv, D.n_scale_tv, D.x_smem_scale, 0);
            ortho(D, 1);
            siblings(D, 1);
            merge(D, 1);
        }
        cur_level_ = -1;
        if (ldlt_ && n_diag_)  // the diag phase (tree.cpp:1621-1624)
            launch("sign_x", [&] {
                sign_x_kernel<T><<<dim3((unsigned)n_diag_, (unsigned)nrhs), 128, 0, s_>>>(ctx_, X, diag_, n_diag_, signs_,
                                                                                       d_xoff_);
            });
        for (int l = P.nlevels - 1; l >= 0; l--) {
            LevelDev& D = levels_[l];
            cur_level_ = l;
            merge(D, 0);
            siblings(D, 0);
            ortho(D, 0);
            cur_count_ = D.n_scale_llt;
            trsv(D.scale_llt, lu_ ? D.scale_inv : D.scale_llt_blk, D.scale_tv, D.n_scale_tv, D.x_smem_scale, 1);
            permx(D.scale_llt, D.n_scale_llt, 0, D.x_smem_scale);
            if (D.n_gb && D.n_gb_tiles)
                launch("gemm_bwd", [&] {
                    if (mr)
                        gemm_mrhs_kernel<T><<<D.n_gb_tiles, 256, 0, s_>>>(ctx_, X, D.gb, D.gbo, D.gb_tiles, 0);
                    else
                        launch_pdl(gemm_bwd2_kernel<T>, dim3(D.n_gb_tiles * nrhs), dim3(256), 0, 1, ctx_, X,
                                     (const DGroup*)D.gb, (const DGemmOp*)D.gbo, (const DTile*)D.gb_tiles,
                                     D.n_gb_tiles, sg, (const long long*)d_xoff_, 0);
                });
            cur_count_ = D.n_elim_llt;
            trsv(D.elim_llt, lu_ ? D.elim_inv : D.elim_llt_blk, D.elim_tv, D.n_elim_tv, D.x_smem_elim, 1);
            permx(D.elim_llt, D.n_elim_llt, 0, D.x_smem_elim);
        }
        cur_level_ = -1;
        launch("perm", [&] {
            launch_pdl(perm_out_kernel<T>, dim3((unsigned)((tot + 255) / 256)), dim3(256), 0, 1, x, ld, X,
                         (const int*)d_perm_, (const long long*)d_slot_, n);
        });
        SPAND_CUDA(cudaGetLastError());
    }

    cudaStream_t s_;
    std::vector<int> perm_h_;
    int dev_;  // the CUDA device of the stream and of every allocation
    std::vector<int> caps_h_;
    const Plan* P_ = nullptr;
    int nc_ = 0;
    std::vector<void*> owned_;
    size_t bytes_ = 0;
    T* arena_ = nullptr;
    T* pristine_ = nullptr;
    long long* d_amap_ = nullptr;
    int64_t amap_n_ = 0;
    double* d_vals_ = nullptr;
    DBlock* d_blk_ = nullptr;
    int* d_cap_ = nullptr;
    int *csize_ = nullptr, *rows0_ = nullptr, *rank_ = nullptr, *cpos_ = nullptr;
    DStatus* status_ = nullptr;
    T* tstore_ = nullptr;
    T *vstore_ = nullptr, *taustore_ = nullptr, *tauws_ = nullptr, *ws_ = nullptr;
    T* ws2_ = nullptr;  // column slabs of the global-memory QRCP
    int *jpvt_ = nullptr, *ipvt_ = nullptr, *colcount_ = nullptr, *fallback_ = nullptr;
    int64_t ws_len_ = 0, cols_len_ = 0;  // elements of ws_ / ws2_ and of jpvt_ / ipvt_
    int items_len_ = 0;                  // entries of fallback_ / colcount_
    int* tv_count_ = nullptr;  // finished row tiles per cluster (triangular products)
    cudaStream_t s2_ = nullptr;  // side stream of the WY factors
    DStatus* h_status_ = nullptr;  // pinned copy of the status word, filled by factorize_enqueue
    cudaEvent_t ev_fork_ = nullptr, ev_join_ = nullptr;
    int* pc_fallback_ = nullptr;  // pivots the cluster Cholesky could not hold
    bool lu_ = false;             // PLU path (general matrices)
    int* lu_perm_ = nullptr;      // per cluster at its solve-slot offset: row permutation of its pivot
    int* lu_swp_ = nullptr;       // and the row interchanges that make it
    int cur_count_ = 0;           // clusters of the pivot op list being applied in the solve
    bool check_launches_ = getenv("SPAND_CHECK_LAUNCHES") != nullptr;
    bool lorasp_ = false;         // LoRaSp plan (explicit siblings with original edges)
    int4* lr_splits_ = nullptr;   // LoRaSp: (block, neighbour, transposed, sibling block)
    // preservation: phi restricted to every hierarchy cluster (capacity x nphi at
    // phioff), its scratch, the natural-order phi, the leaf scatter map, rank1 per cluster
    int nphi_ = 0;
    T *phis_ = nullptr, *phitmp_ = nullptr;
    double* d_phinat_ = nullptr;
    long long *d_phioff_ = nullptr, *d_phidst_ = nullptr;
    int *d_phild_ = nullptr, *rank1_ = nullptr;
    int phi_n_ = 0, phi_alloc_ = 0;
    bool pres_adaptive_ = false;  // preserve + RRQR (tol <= 1) in the running factorization
    bool ldlt_ = false;           // LDLT path (symmetric indefinite)
    T* signs_ = nullptr;          // LDLT: sign(D) of every factored pivot at the cluster's offset
    std::vector<int> diag_h_;     // LDLT: clusters of every ScalingLDLT op (the diag phase)
    int* diag_ = nullptr;
    int n_diag_ = 0, diag_smem_ = 0;
    bool tuned_ = false;
    // re-layered sparsification waves after the first factorization (SPAND_QC_RELAYER=0: the plan's)
    bool relayer_on_ = !(getenv("SPAND_QC_RELAYER") && atoi(getenv("SPAND_QC_RELAYER")) == 0);
    // SPAND_ORTHO_FULL=0: the Orthogonal op of one right-hand side in the blocked form
    bool ortho_full_on_ = !(getenv("SPAND_ORTHO_FULL") && atoi(getenv("SPAND_ORTHO_FULL")) == 0);
    // SPAND_TRSV_SMALL=0: the triangular products of small clusters in row tiles as well
    bool trsv_small_on_ = !(getenv("SPAND_TRSV_SMALL") && atoi(getenv("SPAND_TRSV_SMALL")) == 0);
    // SPAND_TRSM_TC=0: the FP32 panel products on the SIMT kernel
    bool trsm_tc_on_ = !(getenv("SPAND_TRSM_TC") && atoi(getenv("SPAND_TRSM_TC")) == 0);
    // SPAND_TRSM_SMALL=0: the panel products of small pivots a CTA per tile as well
    bool trsm_small_on_ = !(getenv("SPAND_TRSM_SMALL") && atoi(getenv("SPAND_TRSM_SMALL")) == 0);
    // SPAND_SCHUR_TC=0: the FP32 Schur updates on the SIMT kernel
    bool schur_tc_on_ = !(getenv("SPAND_SCHUR_TC") && atoi(getenv("SPAND_SCHUR_TC")) == 0);
    // SPAND_ORTHO_CLUSTER=0: the Orthogonal op of the large clusters on one CTA each
    bool ortho_cluster_on_ = !(getenv("SPAND_ORTHO_CLUSTER") && atoi(getenv("SPAND_ORTHO_CLUSTER")) == 0);
    // SPAND_QC_GLOBAL_PASS=1: queue the global-memory QRCP pass after every wave
    bool gskip_on_ = !(getenv("SPAND_QC_GLOBAL_PASS") && atoi(getenv("SPAND_QC_GLOBAL_PASS")) == 1);
    bool gskip_used_ = false;  // the last factorization left a global pass out
    // SPAND_PDL=0: the solve sweep's kernels launched without programmatic dependence
    bool pdl_on_ = !(getenv("SPAND_PDL") && atoi(getenv("SPAND_PDL")) == 0);
    // SPAND_POTRF_SMALL=0: the pivots of at most 32 rows on the one-CTA kernel as well
    bool potrf_small_on_ = !(getenv("SPAND_POTRF_SMALL") && atoi(getenv("SPAND_POTRF_SMALL")) == 0);
    // a phase's small-cluster and row-tile triangular products in one launch (SPAND_TRSV_FUSE=0: two)
    bool trsv_fuse_on_ = !(getenv("SPAND_TRSV_FUSE") && atoi(getenv("SPAND_TRSV_FUSE")) == 0);
    // register-tiled products in the one-CTA Cholesky and inverse (SPAND_POTRF_TILED=0: one
    // element per thread)
    bool potrf_tiled_on_ = !(getenv("SPAND_POTRF_TILED") && atoi(getenv("SPAND_POTRF_TILED")) == 0);
    // size-class launches of the one-CTA Cholesky (SPAND_POTRF_SPLIT=0: one launch per level)
    bool potrf_split_on_ = !(getenv("SPAND_POTRF_SPLIT") && atoi(getenv("SPAND_POTRF_SPLIT")) == 0);
    // measured QRCP tuning: the factorization after tune_qrcp() times every wave's
    // candidates (SPAND_QC_TUNE=0: the launch model's choice only); the winners are kept per
    // plan fingerprint for the process (trees of the same plan skip the measurement)
    bool measure_on_ = !(getenv("SPAND_QC_TUNE") && atoi(getenv("SPAND_QC_TUNE")) == 0);
    bool measure_next_ = false, measuring_ = false;
    double last_tol_ = 0.0, tuned_tol_ = 0.0;
    std::string tune_key_;
    std::vector<cudaEvent_t> tune_ev_;
    static std::mutex& qc_tune_mutex() {
        static std::mutex m;
        return m;
    }
    static std::map<std::string, std::vector<QcConf>>& qc_tune_cache() {
        static std::map<std::string, std::vector<QcConf>> c;
        return c;
    }
    // the factorization's CUDA graph (SPAND_FACTOR_GRAPH=0: launches one by one)
    bool use_fgraph_ = !(getenv("SPAND_FACTOR_GRAPH") && atoi(getenv("SPAND_FACTOR_GRAPH")) == 0);
    cudaGraph_t fgraph_ = nullptr;
    cudaGraphExec_t fgraph_exec_ = nullptr;
    int64_t fgraph_kernels_ = 0;
    double fgraph_tol_ = -1.0;
    int fgraph_nphi_ = -1;
    int cur_level_ = -1;
    bool scale_phase_ = false;  // the level's scaling pivots (per-level profile names "@S")
    // in-kernel phase timing of the QRCP of one level (SPAND_QC_PROBE=<level>)
    // per-level kernel classes in the profile (SPAND_PROFILE_LEVELS=1)
    bool per_level_ = getenv("SPAND_PROFILE_LEVELS") != nullptr;
    // every sparsification matrix through the global-memory QRCP on full clusters
    // (SPAND_QC_GLOBAL=1; testing and measurement)
    bool force_global_ = getenv("SPAND_QC_GLOBAL") != nullptr;
    // per-wave QRCP classes and a line per wave after tuning (SPAND_PROFILE_LEVELS=2)
    bool per_wave_ = per_level_ && atoi(getenv("SPAND_PROFILE_LEVELS")) >= 2;
    int cur_wave_ = -1;
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

void device_scatter(const double* src, const int* map, int64_t n, double* dst, cudaStream_t s) {
    if (n > 0) scatter_f64_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(src, map, n, dst);
}

void device_pattern_outer(const int* rows, const int* cols, int64_t nnz, const double* lam, const double* x,
                          double* out, cudaStream_t s) {
    if (nnz > 0) pattern_outer_kernel<<<(unsigned)((nnz + 255) / 256), 256, 0, s>>>(nnz, rows, cols, lam, x, out);
}

// Workspace of the device CG, kept across calls for one matrix size.
void PcgWork::release() {
    cudaFree(r); cudaFree(p); cudaFree(z); cudaFree(tmp); cudaFree(partial); cudaFree(sc);
    if (h_sc) cudaFreeHost(h_sc);
    r = p = z = tmp = partial = sc = h_sc = nullptr;
    n = 0;
}

void PcgWork::ensure(int nn) {
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

static thread_local PcgWork g_pcg;

// Preconditioned CG (is.cpp:39-121) with all vectors and scalars on the device; one
// scalar read back per iteration for the stopping test.
PcgResult device_pcg(DeviceFactorBase& M, const DeviceCsr& A, const double* b, double* x, int maxit, double tol,
                     bool use_graph) {
    PcgSystem sys{&M, &A, &g_pcg, b, x};
    device_pcg_batch(&sys, 1, maxit, tol, use_graph);
    return sys.res;
}

// Independent systems advanced in lockstep: every phase of an iteration is queued on all
// systems' streams before the one wait of the iteration (the stopping test of each).
void device_pcg_batch(PcgSystem* sys, int count, int maxit, double tol, bool use_graph) {
    struct St {
        double thr = 0, bb = 0, rr = 0;
        bool active = false;
    };
    std::vector<St> st(count);
    auto L = [&](PcgSystem& q, const char* cls, auto&& f, int k = 1) {
        KernelProfiler& prof = q.M->profiler();
        prof.begin(q.M->stream(), cls);
        f(q.M->stream(), q.A->n, (unsigned)((q.A->n + 255) / 256));
        prof.end(q.M->stream());
        q.M->add_launches(k);
    };
    auto dot = [&](PcgSystem& q, const double* a, const double* bb, int slot) {
        L(q, "dot", [&](cudaStream_t s, int n, unsigned) {
            dot_partial_kernel<<<RED_BLOCKS, RED_THREADS, 0, s>>>(n, a, bb, q.w->partial);
            dot_final_kernel<<<1, RED_THREADS, 0, s>>>(q.w->partial, RED_BLOCKS, q.w->sc + slot);
        }, 2);
    };
    auto spmv = [&](PcgSystem& q, const double* in, double* out) {
        L(q, "spmv", [&](cudaStream_t s, int n, unsigned gb) {
            spmv_kernel<<<gb, 256, 0, s>>>(n, q.A->rowptr, q.A->colind, q.A->val, in, out);
        });
    };
    auto wait_all = [&]() {
        for (int k = 0; k < count; k++)
            if (st[k].active) SPAND_CUDA(cudaStreamSynchronize(sys[k].M->stream()));
    };
    for (int k = 0; k < count; k++) {
        PcgSystem& q = sys[k];
        q.w->ensure(q.A->n);
        q.res = PcgResult{};
        st[k].active = true;
        spmv(q, q.x, q.w->tmp);
        L(q, "axpy", [&](cudaStream_t s, int n, unsigned gb) { sub_kernel<<<gb, 256, 0, s>>>(n, q.b, q.w->tmp, q.w->r); });
        dot(q, q.b, q.b, 4);
        dot(q, q.w->r, q.w->r, 2);
        SPAND_CUDA(cudaMemcpyAsync(q.w->h_sc, q.w->sc, 8 * sizeof(double), cudaMemcpyDeviceToHost, q.M->stream()));
    }
    wait_all();
    for (int k = 0; k < count; k++) {
        PcgSystem& q = sys[k];
        st[k].bb = q.w->h_sc[4];
        if (st[k].bb == 0) {
            SPAND_CUDA(cudaMemsetAsync(q.x, 0, q.A->n * sizeof(double), q.M->stream()));
            SPAND_CUDA(cudaStreamSynchronize(q.M->stream()));
            st[k].active = false;
            continue;
        }
        st[k].thr = tol * tol * st[k].bb;
        st[k].rr = q.w->h_sc[2];
        q.res.relres = std::sqrt(st[k].rr / st[k].bb);
        if (st[k].rr < st[k].thr) {
            st[k].active = false;
            continue;
        }
        SPAND_CUDA(cudaMemcpyAsync(q.w->p, q.w->r, q.A->n * sizeof(double), cudaMemcpyDeviceToDevice, q.M->stream()));
        q.M->solve_device(q.w->p, 1, q.A->n);
        dot(q, q.w->r, q.w->p, 0);
        if (use_graph) q.M->capture_solve(q.w->z, 1, q.A->n);
    }
    int i = 0;
    int live = 0;
    for (int k = 0; k < count; k++) live += st[k].active;
    while (live && i < maxit) {
        for (int k = 0; k < count; k++) {
            if (!st[k].active) continue;
            PcgSystem& q = sys[k];
            spmv(q, q.w->p, q.w->tmp);
            dot(q, q.w->p, q.w->tmp, 1);
            L(q, "axpy", [&](cudaStream_t s, int n, unsigned gb) {
                cg_update_xr_kernel<<<gb, 256, 0, s>>>(n, q.x, q.w->r, q.w->p, q.w->tmp, q.w->sc);
            });
            dot(q, q.w->r, q.w->r, 2);
            SPAND_CUDA(cudaMemcpyAsync(q.w->h_sc + 2, q.w->sc + 2, sizeof(double), cudaMemcpyDeviceToHost,
                                       q.M->stream()));
        }
        wait_all();
        live = 0;
        for (int k = 0; k < count; k++) {
            if (!st[k].active) continue;
            PcgSystem& q = sys[k];
            st[k].rr = q.w->h_sc[2];
            if (st[k].rr < st[k].thr) {
                st[k].active = false;
                q.res.iterations = i + 1;
                q.res.relres = std::sqrt(st[k].rr / st[k].bb);
                continue;
            }
            live++;
            SPAND_CUDA(cudaMemcpyAsync(q.w->z, q.w->r, q.A->n * sizeof(double), cudaMemcpyDeviceToDevice,
                                       q.M->stream()));
            q.M->solve_device(q.w->z, 1, q.A->n);
            L(q, "axpy", [&](cudaStream_t s, int, unsigned) { copy_scalar_kernel<<<1, 1, 0, s>>>(q.w->sc, 3, 0); });
            dot(q, q.w->r, q.w->z, 0);
            L(q, "axpy", [&](cudaStream_t s, int n, unsigned gb) {
                cg_update_p_kernel<<<gb, 256, 0, s>>>(n, q.w->p, q.w->z, q.w->sc);
            });
        }
        i++;
    }
    for (int k = 0; k < count; k++) {
        if (!st[k].active) continue;
        PcgSystem& q = sys[k];
        q.res.iterations = i + 1;
        q.res.relres = std::sqrt(st[k].rr / st[k].bb);
    }
    for (int k = 0; k < count; k++) SPAND_CUDA(cudaGetLastError());
}

// Work buffers of the multi-right-hand-side PCG (n x k operands), grown on demand.
struct PcgMultiWork {
    size_t cap = 0;  // elements per operand
    int kcap = 0;
    double *r = nullptr, *p = nullptr, *z = nullptr, *q = nullptr, *partial = nullptr, *sc = nullptr;
    int* active = nullptr;
    double* h_sc = nullptr;
    int* h_active = nullptr;
    ~PcgMultiWork() { release(); }
    void release() {
        cudaFree(r); cudaFree(p); cudaFree(z); cudaFree(q); cudaFree(partial); cudaFree(sc); cudaFree(active);
        if (h_sc) cudaFreeHost(h_sc);
        if (h_active) cudaFreeHost(h_active);
        r = p = z = q = partial = sc = h_sc = nullptr;
        active = h_active = nullptr;
        cap = 0;
        kcap = 0;
    }
    void ensure(int n, int k) {
        const size_t need = (size_t)n * k;
        if (need <= cap && k <= kcap) return;
        release();
        SPAND_CUDA(cudaMalloc(&r, need * sizeof(double)));
        SPAND_CUDA(cudaMalloc(&p, need * sizeof(double)));
        SPAND_CUDA(cudaMalloc(&z, need * sizeof(double)));
        SPAND_CUDA(cudaMalloc(&q, need * sizeof(double)));
        SPAND_CUDA(cudaMalloc(&partial, (size_t)RED_BLOCKS * k * sizeof(double)));
        SPAND_CUDA(cudaMalloc(&sc, 8 * (size_t)k * sizeof(double)));
        SPAND_CUDA(cudaMalloc(&active, (size_t)k * sizeof(int)));
        SPAND_CUDA(cudaMallocHost(&h_sc, 8 * (size_t)k * sizeof(double)));
        SPAND_CUDA(cudaMallocHost(&h_active, (size_t)k * sizeof(int)));
        cap = need;
        kcap = k;
    }
};

static thread_local PcgMultiWork g_pcgm;

// k independent preconditioned CGs (is.cpp:39-121 per column) advanced in lockstep: one
// SpMV, one multi-right-hand-side preconditioner application and three dots per
// iteration serve every column; a converged column is frozen (its x and r stop changing)
// and keeps its own iteration count.  b, x: n x k, column j at offset j * n.
void device_pcg_multi(DeviceFactorBase& M, const DeviceCsr& A, const double* b, double* x, int k, int maxit,
                      double tol, bool use_graph, int* iters_out, double* relres_out) {
    cudaStream_t s = M.stream();
    KernelProfiler& prof = M.profiler();
    const int n = A.n;
    g_pcgm.ensure(n, k);
    PcgMultiWork& w = g_pcgm;
    auto L = [&](const char* cls, auto&& f, int nk = 1) {
        prof.begin(s, cls);
        f();
        prof.end(s);
        M.add_launches(nk);
    };
    const dim3 gb((unsigned)((n + 255) / 256), (unsigned)k);
    auto dot = [&](const double* a, const double* bb, int slot) {
        L("dot", [&] {
            dot_multi_partial_kernel<<<dim3(RED_BLOCKS, (unsigned)k), RED_THREADS, 0, s>>>(n, a, bb, w.partial);
            dot_multi_final_kernel<<<(unsigned)k, RED_THREADS, 0, s>>>(w.partial, RED_BLOCKS, w.sc, slot);
        }, 2);
    };
    auto spmv = [&](const double* in, double* out) {
        L("spmv", [&] { spmv_multi_kernel<<<gb, 256, 0, s>>>(n, A.rowptr, A.colind, A.val, in, out); });
    };
    spmv(x, w.q);
    L("axpy", [&] { sub_multi_kernel<<<gb, 256, 0, s>>>(n, b, w.q, w.r); });
    dot(b, b, 4);
    dot(w.r, w.r, 2);
    SPAND_CUDA(cudaMemcpyAsync(w.h_sc, w.sc, 8 * (size_t)k * sizeof(double), cudaMemcpyDeviceToHost, s));
    SPAND_CUDA(cudaStreamSynchronize(s));
    std::vector<double> thr(k), bb(k);
    int live = 0;
    for (int j = 0; j < k; j++) {
        bb[j] = w.h_sc[8 * j + 4];
        thr[j] = tol * tol * bb[j];
        const double rr = w.h_sc[8 * j + 2];
        iters_out[j] = 0;
        relres_out[j] = bb[j] > 0 ? std::sqrt(rr / bb[j]) : 0.0;
        w.h_active[j] = (bb[j] > 0 && !(rr < thr[j])) ? 1 : 0;
        if (bb[j] == 0) SPAND_CUDA(cudaMemsetAsync(x + (size_t)j * n, 0, n * sizeof(double), s));
        live += w.h_active[j];
    }
    if (!live) {
        SPAND_CUDA(cudaStreamSynchronize(s));
        return;
    }
    SPAND_CUDA(cudaMemcpyAsync(w.active, w.h_active, (size_t)k * sizeof(int), cudaMemcpyHostToDevice, s));
    SPAND_CUDA(cudaMemcpyAsync(w.p, w.r, (size_t)n * k * sizeof(double), cudaMemcpyDeviceToDevice, s));
    M.solve_device(w.p, k, n);
    dot(w.r, w.p, 0);
    if (use_graph) M.capture_solve(w.z, k, n);
    int i = 0;
    while (i < maxit) {
        spmv(w.p, w.q);
        dot(w.p, w.q, 1);
        L("axpy", [&] { cg_multi_update_xr_kernel<<<gb, 256, 0, s>>>(n, x, w.r, w.p, w.q, w.sc, w.active); });
        dot(w.r, w.r, 2);
        SPAND_CUDA(cudaMemcpyAsync(w.h_sc, w.sc, 8 * (size_t)k * sizeof(double), cudaMemcpyDeviceToHost, s));
        SPAND_CUDA(cudaStreamSynchronize(s));
        live = 0;
        for (int j = 0; j < k; j++) {
            if (!w.h_active[j]) continue;
            const double rr = w.h_sc[8 * j + 2];
            relres_out[j] = std::sqrt(rr / bb[j]);
            if (rr < thr[j]) {
                w.h_active[j] = 0;
                iters_out[j] = i + 1;
            } else {
                live++;
            }
        }
        if (!live) break;
        SPAND_CUDA(cudaMemcpyAsync(w.active, w.h_active, (size_t)k * sizeof(int), cudaMemcpyHostToDevice, s));
        SPAND_CUDA(cudaMemcpyAsync(w.z, w.r, (size_t)n * k * sizeof(double), cudaMemcpyDeviceToDevice, s));
        M.solve_device(w.z, k, n);
        L("axpy", [&] { copy_scalar_multi_kernel<<<(unsigned)((k + 63) / 64), 64, 0, s>>>(w.sc, k, 3, 0); });
        dot(w.r, w.z, 0);
        L("axpy", [&] { cg_multi_update_p_kernel<<<gb, 256, 0, s>>>(n, w.p, w.z, w.sc, w.active); });
        i++;
    }
    for (int j = 0; j < k; j++)
        if (w.h_active[j]) iters_out[j] = i + 1;
    SPAND_CUDA(cudaGetLastError());
    SPAND_CUDA(cudaStreamSynchronize(s));
}


// ------------------------------------------------------------------------------------
// GMRES (is.cpp:123-300): Eigen's restarted GMRES with Householder Arnoldi, left
// preconditioned by M.  The reflectors H_i = I - tau_i u_i u_i^T (u_i: zero above row i,
// one at row i) are the columns of Y (m x (restart+1), FP64, device); their product is
// kept in compact WY form, H_0 H_1 ... H_{k-1} = I - Y_k T_k Y_k^T (T_k upper triangular,
// host), so that each application of the k reflectors of an iteration becomes one
// reduction Y^T v and one update v - Y z instead of k dependent rank-1 steps.  The
// Hessenberg columns, Givens rotations and the small triangular solve stay on the host,
// as small vectors.  Same arithmetic as the sequential reflectors up to rounding.
// ------------------------------------------------------------------------------------
constexpr int GM_BLOCKS = 304;

// partial[b * k + i] = sum over block b's share of rows [r0, m) of Y[r + i ldy] v[r]
__global__ void gm_dots_kernel(int r0, int m, int k, const double* __restrict__ Y, long long ldy,
                               const double* __restrict__ v, double* __restrict__ partial) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const long long len = m - r0;
    const long long span = (len + gridDim.x - 1) / gridDim.x;
    const long long a = r0 + (long long)blockIdx.x * span;
    const long long e = min((long long)m, a + span);
    for (int i = warp; i < k; i += nw) {
        const double* y = Y + (long long)i * ldy;
        double s = 0;
        for (long long r = a + lane; r < e; r += 32) s += y[r] * v[r];
        s = warp_sum(s);
        if (lane == 0) partial[(long long)blockIdx.x * k + i] = s;
    }
}

__global__ void gm_dots_final_kernel(int nb, int k, const double* __restrict__ partial, double* __restrict__ out) {
    const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (i >= k) return;
    double s = 0;
    for (int b = lane; b < nb; b += 32) s += partial[(long long)b * k + i];
    s = warp_sum(s);
    if (lane == 0) out[i] = s;
}

// out[r] = base[r] - sum_{i<k} Y[r + i ldy] z[i]; zy = (z[0..k), y[0..k)).
// mode 0: base = e_unit; 1: base = out; 2: base = out + (r < k ? y[r] : 0)
__global__ void gm_update_kernel(int m, int k, const double* __restrict__ Y, long long ldy,
                                 const double* __restrict__ zy, double* __restrict__ out, int mode, int unit) {
    extern __shared__ double zs[];
    for (int i = threadIdx.x; i < 2 * k; i += blockDim.x) zs[i] = zy[i];
    __syncthreads();
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= m) return;
    double s = 0;
    for (int i = 0; i < k; i++) s += Y[r + i * ldy] * zs[i];
    double base = mode == 0 ? (r == unit ? 1.0 : 0.0) : out[r];
    if (mode == 2 && r < k) base += zs[k + r];
    out[r] = base - s;
}

// column k of Y: zero above row k, one at row k, v[r] / d below (zero when d == 0)
__global__ void gm_reflector_kernel(int m, int k, double* __restrict__ ycol, const double* __restrict__ v, double d) {
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= m) return;
    ycol[r] = r < k ? 0.0 : (r == k ? 1.0 : (d != 0.0 ? v[r] / d : 0.0));
}

namespace {
struct GmGivens {
    double c = 1, s = 0;
};
// G with G^T (p, q) = (r, 0) (Eigen's real JacobiRotation::makeGivens)
GmGivens gm_make_givens(double p, double q) {
    GmGivens g;
    if (q == 0) {
        g.c = p < 0 ? -1 : 1;
        g.s = 0;
    } else if (p == 0) {
        g.c = 0;
        g.s = q < 0 ? 1 : -1;
    } else if (std::fabs(p) > std::fabs(q)) {
        double t = q / p, u = std::sqrt(1 + t * t);
        if (p < 0) u = -u;
        g.c = 1 / u;
        g.s = -t * g.c;
    } else {
        double t = p / q, u = std::sqrt(1 + t * t);
        if (q < 0) u = -u;
        g.s = -1 / u;
        g.c = -t * g.s;
    }
    return g;
}
void gm_rotate(double* v, int i, const GmGivens& g) {
    const double x = v[i], y = v[i + 1];
    v[i] = g.c * x - g.s * y;
    v[i + 1] = g.s * x + g.c * y;
}
}  // namespace

PcgResult device_gmres(DeviceFactorBase& M, const DeviceCsr& A, const double* b, double* x, int maxit, int restart,
                       double tol) {
    const int m = A.n;
    const int R = std::max(1, std::min(restart, m));
    if (2 * (int64_t)(R + 1) * (int64_t)sizeof(double) > 200 * 1024)
        throw DeviceError{SPAND_ERR_UNSUPPORTED, "GMRES restart length above 12799"};
    static std::once_flag attr_once;
    std::call_once(attr_once, [] {
        SPAND_CUDA(cudaFuncSetAttribute(gm_update_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    });
    cudaStream_t s = M.stream();
    PcgResult res;
    const unsigned gb = (unsigned)((m + 255) / 256);
    const int nb = GM_BLOCKS;
    const long long ldy = m;
    // device: two m-vectors, Y, partials, reduction output, z/y; host: pinned scalars
    double *v = nullptr, *t = nullptr, *Y = nullptr, *partial = nullptr, *dout = nullptr, *dzy = nullptr, *hp = nullptr;
    auto cleanup = [&] {
        cudaFree(v); cudaFree(t); cudaFree(Y); cudaFree(partial); cudaFree(dout); cudaFree(dzy);
        if (hp) cudaFreeHost(hp);
    };
    try {
        SPAND_CUDA(cudaMalloc(&v, (size_t)m * sizeof(double)));
        SPAND_CUDA(cudaMalloc(&t, (size_t)m * sizeof(double)));
        SPAND_CUDA(cudaMalloc(&Y, (size_t)m * (R + 1) * sizeof(double)));
        SPAND_CUDA(cudaMalloc(&partial, (size_t)nb * (R + 1) * sizeof(double)));
        SPAND_CUDA(cudaMalloc(&dout, (size_t)(R + 2) * sizeof(double)));
        SPAND_CUDA(cudaMalloc(&dzy, (size_t)2 * (R + 1) * sizeof(double)));
        SPAND_CUDA(cudaMallocHost(&hp, (size_t)4 * (R + 2) * sizeof(double)));
        double* hd = hp;                 // reduction results
        double* hz = hp + (R + 2);       // z, y staged for upload
        double* hv = hp + 3 * (R + 2);   // leading entries of v
        auto launched = [&](int k) { M.add_launches(k); };
        // k dot products Y[:, i] . w over rows [r0, m) -> hd[0..k)
        auto dots = [&](int r0, int k, const double* Yp, long long ld, const double* w) {
            if (k <= 0) return;
            if (r0 >= m) {
                for (int i = 0; i < k; i++) hd[i] = 0;
                return;
            }
            gm_dots_kernel<<<nb, 256, 0, s>>>(r0, m, k, Yp, ld, w, partial);
            gm_dots_final_kernel<<<(unsigned)((k + 7) / 8), 256, 0, s>>>(nb, k, partial, dout);
            launched(2);
            SPAND_CUDA(cudaMemcpyAsync(hd, dout, (size_t)k * sizeof(double), cudaMemcpyDeviceToHost, s));
            SPAND_CUDA(cudaStreamSynchronize(s));
        };
        auto update = [&](int k, double* out, int mode, int unit) {
            SPAND_CUDA(cudaMemcpyAsync(dzy, hz, (size_t)2 * std::max(k, 1) * sizeof(double), cudaMemcpyHostToDevice, s));
            gm_update_kernel<<<gb, 256, (size_t)2 * std::max(k, 1) * sizeof(double), s>>>(m, k, Y, ldy, dzy, out, mode,
                                                                                         unit);
            launched(1);
        };
        dots(0, 1, b, 0, b);
        if (std::sqrt(hd[0]) <= std::numeric_limits<double>::min()) {
            SPAND_CUDA(cudaMemsetAsync(x, 0, (size_t)m * sizeof(double), s));
            SPAND_CUDA(cudaStreamSynchronize(s));
            cleanup();
            res.iterations = 1;
            return res;
        }
        std::vector<double> Ytop((size_t)(R + 1) * (R + 1), 0.0), T((size_t)(R + 1) * (R + 1), 0.0);
        std::vector<double> Hr((size_t)(R + 1) * (R + 1), 0.0), w(R + 1, 0.0), tau(R + 1, 0.0), q(R + 1), z(R + 1);
        std::vector<GmGivens> G(R);
        auto ytop = [&](int i, int r) -> double& { return Ytop[(size_t)i * (R + 1) + r]; };  // Y[r, i], r <= R
        auto Tm = [&](int i, int j) -> double& { return T[(size_t)j * (R + 1) + i]; };
        auto Hc = [&](int i, int j) -> double& { return Hr[(size_t)j * (R + 1) + i]; };
        // reflector k from v[k:] (c0 = v[k]); returns the new v[k]; fills Y column k, its top,
        // tau[k] and column k of T
        auto tail_of = [&](int k) {  // |v[k+1:]|^2
            if (k + 1 >= m) return 0.0;
            dots(k + 1, 1, v, 0, v);
            return hd[0];
        };
        auto new_reflector = [&](int k, double c0, double tail) -> double {
            double beta = c0, d = 0, tk = 0;
            if (tail > std::numeric_limits<double>::min()) {
                beta = std::sqrt(c0 * c0 + tail);
                if (c0 >= 0) beta = -beta;
                d = c0 - beta;
                tk = (beta - c0) / beta;
            }
            gm_reflector_kernel<<<gb, 256, 0, s>>>(m, k, Y + (size_t)k * ldy, v, d);
            launched(1);
            const int top = std::min(R + 1, m);
            SPAND_CUDA(cudaMemcpyAsync(&ytop(k, 0), Y + (size_t)k * ldy, (size_t)top * sizeof(double),
                                       cudaMemcpyDeviceToHost, s));
            SPAND_CUDA(cudaStreamSynchronize(s));
            tau[k] = tk;
            // T_{k+1} = [T_k, -tau_k T_k (Y_k^T u_k); 0, tau_k]
            for (int i = 0; i <= k; i++) Tm(i, k) = 0;
            Tm(k, k) = tk;
            if (k > 0 && tk != 0) {
                dots(0, k, Y, ldy, Y + (size_t)k * ldy);
                for (int i = 0; i < k; i++) {
                    double acc = 0;
                    for (int j = i; j < k; j++) acc += Tm(i, j) * hd[j];
                    Tm(i, k) = -tk * acc;
                }
            }
            // v[k] after H_k: c0 - tau (c0 + ess . v_tail), ess . v_tail = tail / d
            return tk == 0 ? c0 : c0 - tk * (c0 + tail / d);
        };
        double r0norm = -1;
        auto start = [&] {
            device_spmv(A, x, t, s);
            sub_kernel<<<gb, 256, 0, s>>>(m, b, t, v);
            launched(2);
            M.solve_device(v, 1, m);
            if (r0norm < 0) {
                dots(0, 1, v, 0, v);
                r0norm = std::sqrt(hd[0]);
            }
            SPAND_CUDA(cudaMemcpyAsync(hv, v, sizeof(double), cudaMemcpyDeviceToHost, s));
            SPAND_CUDA(cudaStreamSynchronize(s));
            std::fill(w.begin(), w.end(), 0.0);
            std::fill(tau.begin(), tau.end(), 0.0);
            std::fill(Hr.begin(), Hr.end(), 0.0);
            w[0] = new_reflector(0, hv[0], tail_of(0));
        };
        start();
        if (r0norm == 0) {
            cleanup();
            res.iterations = 1;
            return res;
        }
        int it = 0;
        double err = 1.0;
        for (int k = 1; k <= R; ++k) {
            ++it;
            // v = H_0 ... H_{k-1} e_{k-1} = e_{k-1} - Y_k T_k Y_k[k-1, :]^T
            for (int i = 0; i < k; i++) q[i] = ytop(i, k - 1);
            for (int i = 0; i < k; i++) {
                double acc = 0;
                for (int j = i; j < k; j++) acc += Tm(i, j) * q[j];
                hz[i] = acc;
            }
            update(k, v, 0, k - 1);
            device_spmv(A, v, t, s);
            launched(1);
            std::swap(v, t);
            M.solve_device(v, 1, m);
            // v = H_{k-1} ... H_0 v = v - Y_k T_k^T (Y_k^T v)
            dots(0, k, Y, ldy, v);
            for (int i = 0; i < k; i++) {
                double acc = 0;
                for (int j = 0; j <= i; j++) acc += Tm(j, i) * hd[j];
                hz[i] = acc;
            }
            update(k, v, 1, 0);
            const int lead = std::min(k + 1, m);
            SPAND_CUDA(cudaMemcpyAsync(hv, v, (size_t)lead * sizeof(double), cudaMemcpyDeviceToHost, s));
            SPAND_CUDA(cudaStreamSynchronize(s));
            if (k < m) {
                const double tail = tail_of(k);
                if (hv[k] * hv[k] + tail != 0.0) hv[k] = new_reflector(k, hv[k], tail);
                else {
                    tau[k] = 0;
                    gm_reflector_kernel<<<gb, 256, 0, s>>>(m, k, Y + (size_t)k * ldy, v, 0.0);
                    launched(1);
                    for (int r = 0; r <= R; r++) ytop(k, r) = r == k ? 1.0 : 0.0;
                    for (int i = 0; i <= k; i++) Tm(i, k) = 0;
                }
            }
            for (int i = 0; i + 1 < k; ++i) gm_rotate(hv, i, G[i]);
            if (k < m && hv[k] != 0) {
                G[k - 1] = gm_make_givens(hv[k - 1], hv[k]);
                gm_rotate(hv, k - 1, G[k - 1]);
                gm_rotate(w.data(), k - 1, G[k - 1]);
            }
            for (int i = 0; i < k; i++) Hc(i, k - 1) = hv[i];
            err = std::fabs(w[k]) / r0norm;
            const bool stop = (k == m || err < tol || it == maxit);
            if (stop || k == R) {
                // y = R^{-1} w[0:k]; x += H_0 ... H_{k-1} [y; 0] = [y; 0] - Y T (Y[0:k, :]^T y)
                std::vector<double> y(w.begin(), w.begin() + k);
                for (int i = k - 1; i >= 0; i--) {
                    double acc = y[i];
                    for (int j = i + 1; j < k; j++) acc -= Hc(i, j) * y[j];
                    y[i] = acc / Hc(i, i);
                }
                for (int i = 0; i < k; i++) {
                    double acc = 0;
                    for (int r = 0; r < k; r++) acc += ytop(i, r) * y[r];
                    q[i] = acc;
                }
                for (int i = 0; i < k; i++) {
                    double acc = 0;
                    for (int j = i; j < k; j++) acc += Tm(i, j) * q[j];
                    hz[i] = acc;
                    hz[k + i] = y[i];
                }
                update(k, x, 2, 0);
                if (stop) break;
                k = 0;
                start();
            }
        }
        SPAND_CUDA(cudaGetLastError());
        SPAND_CUDA(cudaStreamSynchronize(s));
        res.iterations = it;
        res.relres = err;
    } catch (...) {
        cleanup();
        throw;
    }
    cleanup();
    return res;
}

// v_out = v_in / h
__global__ void gm_scale_kernel(int m, const double* __restrict__ in, double* __restrict__ out, double h) {
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r < m) out[r] = in[r] / h;
}

// Flexible GMRES (no reference counterpart): right preconditioned, z_j = M^{-1} v_j kept,
// Arnoldi on A z_j with classical Gram-Schmidt applied twice, restarted from the true
// residual.  The Arnoldi relation A Z_k = V_{k+1} H_k holds in FP64 whatever precision the
// preconditioner computes in, so the recurrence residual is the true |b - A x| (up to FP64
// rounding) and a reduced-precision factor still reaches an FP64 tolerance.  Stops when
// |b - A x| < tol |b|; relres: that ratio.
PcgResult device_fgmres(DeviceFactorBase& M, const DeviceCsr& A, const double* b, double* x, int maxit, int restart,
                        double tol) {
    const int m = A.n;
    const int R = std::max(1, std::min(restart, m));
    if (2 * (int64_t)(R + 1) * (int64_t)sizeof(double) > 200 * 1024)
        throw DeviceError{SPAND_ERR_UNSUPPORTED, "FGMRES restart length above 12799"};
    static std::once_flag attr_once;
    std::call_once(attr_once, [] {
        SPAND_CUDA(cudaFuncSetAttribute(gm_update_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    });
    cudaStream_t s = M.stream();
    PcgResult res;
    const unsigned gb = (unsigned)((m + 255) / 256);
    const int nb = GM_BLOCKS;
    const long long ld = m;
    double *V = nullptr, *Z = nullptr, *w = nullptr, *partial = nullptr, *dout = nullptr, *dzy = nullptr, *hp = nullptr;
    auto cleanup = [&] {
        cudaFree(V); cudaFree(Z); cudaFree(w); cudaFree(partial); cudaFree(dout); cudaFree(dzy);
        if (hp) cudaFreeHost(hp);
    };
    try {
        SPAND_CUDA(cudaMalloc(&V, (size_t)m * (R + 1) * sizeof(double)));
        SPAND_CUDA(cudaMalloc(&Z, (size_t)m * R * sizeof(double)));
        SPAND_CUDA(cudaMalloc(&w, (size_t)m * sizeof(double)));
        SPAND_CUDA(cudaMalloc(&partial, (size_t)nb * (R + 1) * sizeof(double)));
        SPAND_CUDA(cudaMalloc(&dout, (size_t)(R + 2) * sizeof(double)));
        SPAND_CUDA(cudaMalloc(&dzy, (size_t)2 * (R + 1) * sizeof(double)));
        SPAND_CUDA(cudaMallocHost(&hp, (size_t)3 * (R + 2) * sizeof(double)));
        double* hd = hp;
        double* hz = hp + (R + 2);
        auto dots = [&](int k, const double* Yp, long long ldy, const double* v) {
            gm_dots_kernel<<<nb, 256, 0, s>>>(0, m, k, Yp, ldy, v, partial);
            gm_dots_final_kernel<<<(unsigned)((k + 7) / 8), 256, 0, s>>>(nb, k, partial, dout);
            M.add_launches(2);
            SPAND_CUDA(cudaMemcpyAsync(hd, dout, (size_t)k * sizeof(double), cudaMemcpyDeviceToHost, s));
            SPAND_CUDA(cudaStreamSynchronize(s));
        };
        auto update = [&](int k, const double* Yp, double* out, int mode) {
            SPAND_CUDA(cudaMemcpyAsync(dzy, hz, (size_t)2 * std::max(k, 1) * sizeof(double), cudaMemcpyHostToDevice, s));
            gm_update_kernel<<<gb, 256, (size_t)2 * std::max(k, 1) * sizeof(double), s>>>(m, k, Yp, ld, dzy, out,
                                                                                         mode, 0);
            M.add_launches(1);
        };
        dots(1, b, 0, b);
        const double bnorm = std::sqrt(hd[0]);
        if (bnorm == 0) {
            SPAND_CUDA(cudaMemsetAsync(x, 0, (size_t)m * sizeof(double), s));
            SPAND_CUDA(cudaStreamSynchronize(s));
            cleanup();
            return res;
        }
        std::vector<double> H((size_t)(R + 1) * R, 0.0), g(R + 1), y(R);
        std::vector<GmGivens> G(R);
        auto Hc = [&](int i, int j) -> double& { return H[(size_t)j * (R + 1) + i]; };
        int it = 0;
        double err = 1.0;
        while (true) {
            // v_0 = r / |r|, r = b - A x (FP64)
            device_spmv(A, x, w, s);
            sub_kernel<<<gb, 256, 0, s>>>(m, b, w, w);
            M.add_launches(2);
            dots(1, w, 0, w);
            const double beta = std::sqrt(hd[0]);
            err = beta / bnorm;
            if (err < tol || it >= maxit || beta == 0) break;
            gm_scale_kernel<<<gb, 256, 0, s>>>(m, w, V, beta);
            M.add_launches(1);
            std::fill(g.begin(), g.end(), 0.0);
            g[0] = beta;
            int k = 0;
            for (; k < R && it < maxit;) {
                double* zk = Z + (size_t)k * ld;
                SPAND_CUDA(cudaMemcpyAsync(zk, V + (size_t)k * ld, (size_t)m * sizeof(double), cudaMemcpyDeviceToDevice,
                                           s));
                M.solve_device(zk, 1, m);
                device_spmv(A, zk, w, s);
                M.add_launches(1);
                // classical Gram-Schmidt, twice
                for (int i = 0; i <= k; i++) Hc(i, k) = 0;
                for (int pass = 0; pass < 2; pass++) {
                    dots(k + 1, V, ld, w);
                    for (int i = 0; i <= k; i++) {
                        hz[i] = hd[i];
                        Hc(i, k) += hd[i];
                    }
                    update(k + 1, V, w, 1);
                }
                dots(1, w, 0, w);
                const double h = std::sqrt(hd[0]);
                Hc(k + 1, k) = h;
                if (h != 0) {
                    gm_scale_kernel<<<gb, 256, 0, s>>>(m, w, V + (size_t)(k + 1) * ld, h);
                    M.add_launches(1);
                }
                for (int i = 0; i < k; i++) {
                    double col[2] = {Hc(i, k), Hc(i + 1, k)};
                    gm_rotate(col, 0, G[i]);
                    Hc(i, k) = col[0];
                    Hc(i + 1, k) = col[1];
                }
                G[k] = gm_make_givens(Hc(k, k), Hc(k + 1, k));
                {
                    double col[2] = {Hc(k, k), Hc(k + 1, k)};
                    gm_rotate(col, 0, G[k]);
                    Hc(k, k) = col[0];
                    Hc(k + 1, k) = 0;
                }
                gm_rotate(g.data(), k, G[k]);
                ++it;
                ++k;
                err = std::fabs(g[k]) / bnorm;
                if (err < tol || h == 0) break;
            }
            // x += Z_k y, y = R^{-1} g[0:k]
            for (int i = k - 1; i >= 0; i--) {
                double acc = g[i];
                for (int j = i + 1; j < k; j++) acc -= Hc(i, j) * y[j];
                y[i] = acc / Hc(i, i);
            }
            for (int i = 0; i < k; i++) hz[i] = -y[i];
            update(k, Z, x, 1);
            if (err < tol || it >= maxit) {
                // the true residual decides; the loop head recomputes it
                device_spmv(A, x, w, s);
                sub_kernel<<<gb, 256, 0, s>>>(m, b, w, w);
                M.add_launches(2);
                dots(1, w, 0, w);
                err = std::sqrt(hd[0]) / bnorm;
                if (err < tol || it >= maxit) break;
            }
        }
        SPAND_CUDA(cudaGetLastError());
        SPAND_CUDA(cudaStreamSynchronize(s));
        res.iterations = it;
        res.relres = err;
    } catch (...) {
        cleanup();
        throw;
    }
    cleanup();
    return res;
}

// Iterative refinement (is.cpp:12-37): x += M^{-1} (b - A x) until |b - A x| < tol |b|.
PcgResult device_ir(DeviceFactorBase& M, const DeviceCsr& A, const double* b, double* x, int maxit, double tol) {
    const int n = A.n;
    cudaStream_t s = M.stream();
    PcgWork& w = g_pcg;
    w.ensure(n);
    const unsigned gb = (unsigned)((n + 255) / 256);
    auto dot = [&](const double* a, const double* c) {
        dot_partial_kernel<<<RED_BLOCKS, RED_THREADS, 0, s>>>(n, a, c, w.partial);
        dot_final_kernel<<<1, RED_THREADS, 0, s>>>(w.partial, RED_BLOCKS, w.sc);
        M.add_launches(2);
        SPAND_CUDA(cudaMemcpyAsync(w.h_sc, w.sc, sizeof(double), cudaMemcpyDeviceToHost, s));
        SPAND_CUDA(cudaStreamSynchronize(s));
        return w.h_sc[0];
    };
    auto residual = [&] {
        device_spmv(A, x, w.tmp, s);
        sub_kernel<<<gb, 256, 0, s>>>(n, b, w.tmp, w.r);
        M.add_launches(2);
    };
    PcgResult res;
    residual();
    const double bb = dot(b, b);
    if (bb == 0) {
        SPAND_CUDA(cudaMemsetAsync(x, 0, (size_t)n * sizeof(double), s));
        SPAND_CUDA(cudaStreamSynchronize(s));
        return res;
    }
    const double thr = tol * tol * bb;
    double rr = dot(w.r, w.r);
    int i = 1;
    while (rr >= thr && i < maxit) {
        M.solve_device(w.r, 1, n);
        axpy_kernel<<<gb, 256, 0, s>>>(n, 1.0, w.r, x);
        M.add_launches(1);
        residual();
        rr = dot(w.r, w.r);
        if (rr < thr) break;
        i++;
    }
    SPAND_CUDA(cudaGetLastError());
    res.iterations = i;
    res.relres = std::sqrt(rr / bb);
    return res;
}


// ------------------------------------------------------------------------------------
// Segmented PCG: independent systems stored as consecutive segments of one vector
// (system s = rows [off[s], off[s+1])) and preconditioned by one factor of their
// block-diagonal matrix.  Each system follows cg (is.cpp:39-121) with its own scalars; one
// SpMV, one preconditioner application and per-segment dots serve all systems per
// iteration, and a converged system's x, r and p stop changing.
// ------------------------------------------------------------------------------------
__global__ void seg_dot_kernel(const long long* __restrict__ off, const double* __restrict__ a,
                               const double* __restrict__ b, double* __restrict__ out) {
    __shared__ double red[33];
    const int s = blockIdx.x;
    const long long lo = off[s], hi = off[s + 1];
    double acc = 0;
    for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) acc += a[i] * b[i];
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) out[s] = acc;
}

// x += alpha_s p, r -= alpha_s Ap with alpha_s = rz[s] / pAp[s]
__global__ void seg_update_xr_kernel(int n, const int* __restrict__ seg, double* __restrict__ x,
                                     double* __restrict__ r, const double* __restrict__ p,
                                     const double* __restrict__ Ap, const double* __restrict__ rz,
                                     const double* __restrict__ pAp, const int* __restrict__ active) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = seg[i];
    if (!active[s]) return;
    const double alpha = rz[s] / pAp[s];
    x[i] += alpha * p[i];
    r[i] -= alpha * Ap[i];
}

// p = z + beta_s p with beta_s = rz[s] / rz_old[s]
__global__ void seg_update_p_kernel(int n, const int* __restrict__ seg, double* __restrict__ p,
                                    const double* __restrict__ z, const double* __restrict__ rz,
                                    const double* __restrict__ rz_old, const int* __restrict__ active) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = seg[i];
    if (!active[s]) return;
    p[i] = z[i] + (rz[s] / rz_old[s]) * p[i];
}

void SegPcgWork::release() {
    cudaFree(r); cudaFree(p); cudaFree(z); cudaFree(Ap); cudaFree(sc); cudaFree(active);
    if (h_sc) cudaFreeHost(h_sc);
    if (h_active) cudaFreeHost(h_active);
    r = p = z = Ap = sc = h_sc = nullptr;
    active = h_active = nullptr;
    n = 0;
    k = 0;
}

void SegPcgWork::ensure(int nn, int kk) {
    if (nn == n && kk == k) return;
    release();
    SPAND_CUDA(cudaMalloc(&r, (size_t)nn * sizeof(double)));
    SPAND_CUDA(cudaMalloc(&p, (size_t)nn * sizeof(double)));
    SPAND_CUDA(cudaMalloc(&z, (size_t)nn * sizeof(double)));
    SPAND_CUDA(cudaMalloc(&Ap, (size_t)nn * sizeof(double)));
    SPAND_CUDA(cudaMalloc(&sc, (size_t)5 * kk * sizeof(double)));
    SPAND_CUDA(cudaMalloc(&active, (size_t)kk * sizeof(int)));
    SPAND_CUDA(cudaMallocHost(&h_sc, (size_t)5 * kk * sizeof(double)));
    SPAND_CUDA(cudaMallocHost(&h_active, (size_t)kk * sizeof(int)));
    n = nn;
    k = kk;
}

void device_pcg_segmented(DeviceFactorBase& M, const DeviceCsr& A, const double* b, double* x, int nseg,
                          const long long* off, const long long* off_host, const int* seg, SegPcgWork& w, int maxit,
                          double tol, int* iters_out, double* relres_out) {
    const int n = A.n, K = nseg;
    cudaStream_t s = M.stream();
    w.ensure(n, K);
    const unsigned gb = (unsigned)((n + 255) / 256);
    // scalars: rz, rz_old, pAp, rr, bb (K each)
    double *rz = w.sc, *rz_old = w.sc + K, *pAp = w.sc + 2 * K, *rr = w.sc + 3 * K, *bb = w.sc + 4 * K;
    auto L = [&](const char* cls, auto&& f, int k = 1) {
        KernelProfiler& prof = M.profiler();
        prof.begin(s, cls);
        f();
        prof.end(s);
        M.add_launches(k);
    };
    auto dot = [&](const double* a, const double* c, double* out) {
        L("dot", [&] { seg_dot_kernel<<<K, 512, 0, s>>>(off, a, c, out); });
    };
    auto read = [&](const double* src, int count) {
        SPAND_CUDA(cudaMemcpyAsync(w.h_sc, src, (size_t)count * sizeof(double), cudaMemcpyDeviceToHost, s));
        SPAND_CUDA(cudaStreamSynchronize(s));
    };
    std::vector<double> thr(K), bbh(K);
    std::vector<char> done(K, 0);
    device_spmv(A, x, w.Ap, s);
    L("axpy", [&] { sub_kernel<<<gb, 256, 0, s>>>(n, b, w.Ap, w.r); }, 2);
    dot(b, b, bb);
    dot(w.r, w.r, rr);
    read(rr, 2 * K);  // rr, bb
    int live = 0;
    for (int j = 0; j < K; j++) {
        bbh[j] = w.h_sc[K + j];
        const double r2 = w.h_sc[j];
        iters_out[j] = 0;
        relres_out[j] = 0;
        w.h_active[j] = 0;
        if (bbh[j] == 0) {  // zero right-hand side: x = 0 (is.cpp:55-60)
            SPAND_CUDA(cudaMemsetAsync(x + off_host[j], 0, (size_t)(off_host[j + 1] - off_host[j]) * sizeof(double), s));
            done[j] = 1;
            continue;
        }
        thr[j] = tol * tol * bbh[j];
        relres_out[j] = std::sqrt(r2 / bbh[j]);
        if (r2 < thr[j]) {
            done[j] = 1;
            continue;
        }
        w.h_active[j] = 1;
        live++;
    }
    if (!live) {
        SPAND_CUDA(cudaStreamSynchronize(s));
        return;
    }
    SPAND_CUDA(cudaMemcpyAsync(w.active, w.h_active, (size_t)K * sizeof(int), cudaMemcpyHostToDevice, s));
    SPAND_CUDA(cudaMemcpyAsync(w.p, w.r, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    M.solve_device(w.p, 1, n);
    dot(w.r, w.p, rz);
    int i = 0;
    while (i < maxit) {
        device_spmv(A, w.p, w.Ap, s);
        M.add_launches(1);
        dot(w.p, w.Ap, pAp);
        L("axpy", [&] { seg_update_xr_kernel<<<gb, 256, 0, s>>>(n, seg, x, w.r, w.p, w.Ap, rz, pAp, w.active); });
        dot(w.r, w.r, rr);
        read(rr, K);
        live = 0;
        for (int j = 0; j < K; j++) {
            if (!w.h_active[j]) continue;
            relres_out[j] = std::sqrt(w.h_sc[j] / bbh[j]);
            if (w.h_sc[j] < thr[j]) {
                w.h_active[j] = 0;
                iters_out[j] = i + 1;
            } else {
                live++;
            }
        }
        if (!live) break;
        SPAND_CUDA(cudaMemcpyAsync(w.active, w.h_active, (size_t)K * sizeof(int), cudaMemcpyHostToDevice, s));
        SPAND_CUDA(cudaMemcpyAsync(w.z, w.r, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        M.solve_device(w.z, 1, n);
        SPAND_CUDA(cudaMemcpyAsync(rz_old, rz, (size_t)K * sizeof(double), cudaMemcpyDeviceToDevice, s));
        dot(w.r, w.z, rz);
        L("axpy", [&] { seg_update_p_kernel<<<gb, 256, 0, s>>>(n, seg, w.p, w.z, rz, rz_old, w.active); });
        i++;
    }
    for (int j = 0; j < K; j++)
        if (w.h_active[j]) iters_out[j] = i + 1;
    SPAND_CUDA(cudaGetLastError());
    SPAND_CUDA(cudaStreamSynchronize(s));
}

}  // namespace spand

// Preservation kernels (preserve.cuh).  Every matrix here is small and dense and lives in
// global memory (L2-resident); one CTA works on one cluster, its warps on columns.
#include "preserve.cuh"

namespace spand {

constexpr int PV_THREADS = 256;

// Relative size below which the part of a column left by the previous reflectors counts
// as zero (the oracle's rule, QR_DEAD there; FP32: its rounding level).
template <typename T>
__device__ __forceinline__ T qr_dead() {
    return sizeof(T) == 8 ? T(1e-10) : T(1e-4);
}

// Householder QR without pivoting of an m x n matrix in place (LAPACK dgeqr2), n <= m:
// reflector i is [1; A(i+1:m, i)], tau[i]; R on and above the diagonal.  beta =
// -sign(alpha) |(alpha, x)| with sign(-0) = +1, as in the QRCP kernel and the oracle.  A
// column whose remaining part A(i:m, i) is below qr_dead() of its norm depends on the
// previous ones: tau = 0 and the column is left as it is (the oracle's rule; dgeqr2 would
// build that reflector from rounding noise).  Two barriers per column: after the norms
// (both sums in one pass, per-warp partials in red[0:8] and red[16:24]) and after the
// update of the trailing columns; the scaling of column i needs none, since no later
// step reads it.
template <typename T>
__device__ void cta_geqrf(T* A, int lda, int m, int n, T* tau, T* red) {
    const int tid = threadIdx.x, nth = blockDim.x, lane = tid & 31, w = tid >> 5, nw = nth >> 5;
    const int k = min(m, n);
    for (int i = 0; i < k; i++) {
        T* ci = A + (size_t)i * lda;
        T part = 0, head = 0;
        for (int r = i + 1 + tid; r < m; r += nth) part += ci[r] * ci[r];
        for (int r = tid; r < i; r += nth) head += ci[r] * ci[r];
        part = warp_sum(part);
        head = warp_sum(head);
        if (lane == 0) {
            red[w] = part;
            red[16 + w] = head;
        }
        __syncthreads();  // partial norms; the previous step's updates of column i
        T x2 = 0, h2 = 0;
        for (int q = 0; q < nw; q++) {
            x2 += red[q];
            h2 += red[16 + q];
        }
        const T xnorm = dsqrt(x2);
        const T alpha = ci[i];
        const bool dead = dsqrt(alpha * alpha + x2) <= qr_dead<T>() * dsqrt(h2 + alpha * alpha + x2);
        T beta = alpha, tu = 0, sc = 0;
        if (xnorm != T(0) && !dead) {
            beta = alpha >= T(0) ? -hypot(alpha, xnorm) : hypot(alpha, xnorm);
            tu = (beta - alpha) / beta;
            sc = T(1) / (alpha - beta);
        }
        // H = I - tu v v^T, v = [1; sc * x] with x = A(i+1:m, i) still unscaled
        if (tu != T(0))
            for (int j = i + 1 + w; j < n; j += nw) {
                T* cj = A + (size_t)j * lda;
                T s = 0;
                for (int r = i + 1 + lane; r < m; r += 32) s += ci[r] * cj[r];
                s = warp_sum(s);
                const T cji = cj[i];
                __syncwarp();
                const T wv = tu * (cji + sc * s);
                const T cr = wv * sc;
                if (lane == 0) cj[i] = cji - wv;
                for (int r = i + 1 + lane; r < m; r += 32) cj[r] -= cr * ci[r];
            }
        __syncthreads();  // every warp has read the unscaled column and red[]
        if (tid == 0) {
            tau[i] = tu;
            ci[i] = beta;
        }
        if (tu != T(0))
            for (int r = i + 1 + tid; r < m; r += nth) ci[r] *= sc;
    }
    __syncthreads();
}

// The first k columns of Q = H_0 ... H_{k-1} in place over the reflectors of an m x k
// matrix (LAPACK dorg2r: reflectors applied last to first, column i finished at step i).
template <typename T>
__device__ void cta_orgqr(T* A, int lda, int m, int k, const T* tau) {
    const int tid = threadIdx.x, nth = blockDim.x, lane = tid & 31, w = tid >> 5, nw = nth >> 5;
    for (int i = k - 1; i >= 0; i--) {
        T* ci = A + (size_t)i * lda;
        const T ti = tau[i];
        if (i < k - 1 && ti != T(0))
            for (int j = i + 1 + w; j < k; j += nw) {
                T* cj = A + (size_t)j * lda;
                T s = 0;
                for (int r = i + 1 + lane; r < m; r += 32) s += ci[r] * cj[r];
                s = warp_sum(s);
                const T cji = cj[i];
                __syncwarp();
                const T wv = ti * (cji + s);
                if (lane == 0) cj[i] = cji - wv;
                for (int r = i + 1 + lane; r < m; r += 32) cj[r] -= wv * ci[r];
            }
        __syncthreads();
        for (int r = i + 1 + tid; r < m; r += nth) ci[r] *= -ti;
        for (int r = tid; r < i; r += nth) ci[r] = T(0);
        if (tid == 0) ci[i] = T(1) - ti;
        __syncthreads();
    }
}

template <typename T>
__global__ void phi_init_kernel(PhiCtx<T> P, const double* __restrict__ phinat, int n,
                                const int* __restrict__ perm, const long long* __restrict__ dst,
                                const int* __restrict__ ld) {
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= (long long)n * P.nphi) return;
    const int q = (int)(idx % n), j = (int)(idx / n);
    P.phis[dst[q] + (long long)j * ld[q]] = (T)phinat[perm[q] + (long long)j * n];
}

template <typename T>
__global__ void __launch_bounds__(PV_THREADS) phi_scale_kernel(Ctx<T> c, PhiCtx<T> P, T* tmp,
                                                               const int* __restrict__ clusters,
                                                               const int* __restrict__ pivots,
                                                               const int* __restrict__ perm_store,
                                                               const long long* __restrict__ poff) {
    if (c.status->not_spd) return;
    const int cl = clusters[blockIdx.x];
    const int n = c.csize[cl], ld = c.cap[cl], nphi = P.nphi;
    const T* L = bptr(c, pivots[blockIdx.x]);
    const int lld = c.blk[pivots[blockIdx.x]].ld;
    T* F = P.phis + P.off[cl];
    T* X = tmp + P.off[cl];
    const int* perm = perm_store ? perm_store + poff[cl] : nullptr;
    for (int idx = threadIdx.x; idx < n * nphi; idx += blockDim.x) {
        const int i = idx % n, j = idx / n;
        X[i + (size_t)j * ld] = F[(perm ? perm[i] : i) + (size_t)j * ld];
    }
    __syncthreads();
    // F(i, j) = sum_{k >= i} L(k, i) X(k, j), k ascending (the reference's dtrmm order)
    for (int idx = threadIdx.x; idx < n * nphi; idx += blockDim.x) {
        const int i = idx % n, j = idx / n;
        const T* li = L + (size_t)i * lld;
        const T* xj = X + (size_t)j * ld;
        T t = xj[i] * li[i];
        for (int k = i + 1; k < n; k++) t += li[k] * xj[k];
        F[i + (size_t)j * ld] = t;
    }
}

template <typename T>
__global__ void __launch_bounds__(PV_THREADS) phi_merge_kernel(Ctx<T> c, PhiCtx<T> P,
                                                               const int* __restrict__ parents,
                                                               const int* __restrict__ child_ptr,
                                                               const int* __restrict__ child_idx,
                                                               const int* __restrict__ cpos) {
    if (c.status->not_spd) return;
    const int par = parents[blockIdx.x];
    T* Fp = P.phis + P.off[par];
    const int ldp = c.cap[par];
    for (int k = child_ptr[blockIdx.x]; k < child_ptr[blockIdx.x + 1]; k++) {
        const int ch = child_idx[k];
        const int m = c.csize[ch], r0 = cpos[ch], ldc = c.cap[ch];
        const T* Fc = P.phis + P.off[ch];
        for (int idx = threadIdx.x; idx < m * P.nphi; idx += blockDim.x) {
            const int i = idx % m, j = idx / m;
            Fp[r0 + i + (size_t)j * ldp] = Fc[i + (size_t)j * ldc];
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(PV_THREADS) preserve_basis_kernel(Ctx<T> c, PhiCtx<T> P,
                                                                    const DSpars* __restrict__ items,
                                                                    const DAsn* __restrict__ pieces,
                                                                    const T* __restrict__ signs,
                                                                    const long long* __restrict__ soff, T* vstore,
                                                                    T* tauws, int* rank1_out, int* rank_out,
                                                                    int adaptive) {
    __shared__ T red[33];
    if (c.status->not_spd) return;
    const DSpars it = items[blockIdx.x];
    const int cl = it.cluster;
    const int rows = c.csize[cl], nphi = P.nphi;
    const int cols = nphi * (it.count + 1);
    if (cols >= rows) {  // [A_sn phi, phi] spans everything: nothing to compress
        if (threadIdx.x == 0) {
            rank_out[cl] = rows;
            if (adaptive) rank1_out[cl] = rows;
        }
        return;
    }
    const int ld = c.cap[cl];
    const int tid = threadIdx.x, nth = blockDim.x, lane = tid & 31, w = tid >> 5, nw = nth >> 5;
    T* V = vstore + it.v_off;
    const T* Fs = P.phis + P.off[cl];
    // column groups: in-edges (untransposed pieces, listed first), the pivot, out-edges
    int nin = 0;
    while (nin < it.count && !pieces[it.first + nin].transposed) nin++;
    for (int g = 0; g <= it.count; g++) {
        T* D = V + (size_t)g * nphi * ld;
        if (g == nin) {  // pivot: I (LLT) or diag(sign D) (LDLT)
            const T* sg = signs ? signs + soff[cl] : nullptr;
            for (int idx = tid; idx < rows * nphi; idx += nth) {
                const int i = idx % rows, q = idx / rows;
                const T f = Fs[i + (size_t)q * ld];
                D[i + (size_t)q * ld] = sg ? sg[i] * f : f;
            }
            continue;
        }
        const DAsn pc = pieces[it.first + (g < nin ? g : g - 1)];
        const int n = c.csize[pc.nbr], ldn = c.cap[pc.nbr];
        const T* B = bptr(c, pc.block);
        const int bld = c.blk[pc.block].ld;
        const T* Fn = P.phis + P.off[pc.nbr];
        if (!pc.transposed) {  // A_sn (rows x n) phi_n
            for (int idx = tid; idx < rows * nphi; idx += nth) {
                const int i = idx % rows, q = idx / rows;
                const T* f = Fn + (size_t)q * ldn;
                T s = 0;
                for (int k = 0; k < n; k++) s += B[i + (size_t)k * bld] * f[k];
                D[i + (size_t)q * ld] = s;
            }
        } else {  // A_ns^T phi_n, A_ns: n x rows
            for (int pr = w; pr < rows * nphi; pr += nw) {
                const int i = pr % rows, q = pr / rows;
                const T* b = B + (size_t)i * bld;
                const T* f = Fn + (size_t)q * ldn;
                T s = 0;
                for (int k = lane; k < n; k += 32) s += b[k] * f[k];
                s = warp_sum(s);
                if (lane == 0) D[i + (size_t)q * ld] = s;
            }
        }
    }
    __syncthreads();
    T* tau = tauws + it.tau_off;
    cta_geqrf(V, ld, rows, cols, tau, red);
    if (adaptive) {
        cta_orgqr(V, ld, rows, cols, tau);
        if (tid == 0) rank1_out[cl] = cols;
    } else if (tid == 0) {
        rank_out[cl] = cols;
    }
}

template <typename T>
__global__ void __launch_bounds__(PV_THREADS) preserve_combine_kernel(Ctx<T> c, const DSpars* __restrict__ items,
                                                                      const T* ws, T* vstore, T* tauws,
                                                                      const int* __restrict__ rank1_in,
                                                                      int* rank) {
    __shared__ T red[33];
    __shared__ int s_r2;
    if (c.status->not_spd) return;
    const DSpars it = items[blockIdx.x];
    const int cl = it.cluster;
    const int rows = c.csize[cl];
    const int r1 = rank1_in[cl];
    if (threadIdx.x == 0) s_r2 = rank[cl];
    __syncthreads();
    const int r2 = s_r2;
    if (r1 >= rows || r1 + r2 >= rows) {
        if (threadIdx.x == 0) rank[cl] = rows;
        return;
    }
    const int k = r1 + r2, ld = c.cap[cl];
    T* V = vstore + it.v_off;
    const T* W = ws + it.ws_off;  // the QRCP's output, LAPACK column order, ld = cap
    T* tau = tauws + it.tau_off;
    for (int idx = threadIdx.x; idx < rows * r2; idx += blockDim.x) {
        const int i = idx % rows, j = idx / rows;
        V[i + (size_t)(r1 + j) * ld] = W[i + (size_t)j * ld];
    }
    __syncthreads();
    cta_orgqr(V + (size_t)r1 * ld, ld, rows, r2, tau);  // Q2 (its taus are the QRCP's)
    cta_geqrf(V, ld, rows, k, tau, red);                // QR of [Q1 Q2]
    if (threadIdx.x == 0) rank[cl] = k;
}

// Q^T on a tile of up to 32 vectors (a 32-column tile of an in-edge block, a 32-row tile
// of an out-edge block, or phi's columns), in the blocked compact WY form the solve uses
// (blocks of QB = 32 reflectors, T_b upper triangular at the item's v_off in tstore, ld =
// cap): per block b, W = V_b^T X, Y = T_b^T W, X -= V_b Y, blocks in increasing order
// (Q^T = Q_{nb-1}^T ... Q_0^T).  X stays in global memory and passes through shared memory
// PW_KC rows at a time; element (r, l) of the tile is base[r * sr + l * sv].
constexpr int PW_KC = 32;
constexpr int PW_QB = 32;

// Shared memory of one tile application
template <typename T>
struct WyTile {
    T vt[PW_KC][PW_QB + 1];
    T xs[PW_KC][PW_QB + 1];
    T Wm[PW_QB][PW_QB + 1];
    T Ym[PW_QB][PW_QB + 1];
};

// x <- Q^T x on the tile's nv vectors, element (r, l) at base[r * sr + l * sv], r < rows; Q:
// k reflectors in V (ld), T factors in Tm.  Ends with a barrier.
template <typename T>
__device__ void wy_qt_tile(const T* V, const T* Tm, int ld, int rows, int k, T* base, long long sr, long long sv,
                           int nv, WyTile<T>& S) {
    const int tid = threadIdx.x, nth = blockDim.x, lane = tid & 31, w = tid >> 5;
    const bool rfast = sr == 1;  // consecutive threads on consecutive rows (coalesced)
    auto stage = [&](int rb, int i0, int bw) {
        for (int idx = tid; idx < PW_KC * PW_QB; idx += nth) {
            const int kk = idx % PW_KC, ii = idx / PW_KC;
            const int r = rb + kk, col = i0 + ii;
            T v = T(0);
            if (ii < bw && r < rows) v = r > col ? V[r + (size_t)col * ld] : (r == col ? T(1) : T(0));
            S.vt[kk][ii] = v;
            const int rr = rfast ? kk : idx / PW_QB, l = rfast ? ii : idx % PW_QB;
            const int r2 = rb + rr;
            S.xs[rr][l] = (l < nv && r2 < rows) ? base[r2 * sr + l * sv] : T(0);
        }
    };
    const int nb = (k + PW_QB - 1) / PW_QB;
    for (int b = 0; b < nb; b++) {
        const int i0 = b * PW_QB, bw = min(PW_QB, k - i0);
        // W[i][l] = sum_{r >= i0 + i} v_i[r] X[r][l]   (v_i[i0 + i] = 1)
        T acc[4] = {T(0), T(0), T(0), T(0)};
        for (int rb = i0; rb < rows; rb += PW_KC) {
            __syncthreads();
            stage(rb, i0, bw);
            __syncthreads();
            const int kw = min(PW_KC, rows - rb);
            for (int kk = 0; kk < kw; kk++) {
                const T xv = S.xs[kk][lane];
#pragma unroll
                for (int u = 0; u < 4; u++) acc[u] += S.vt[kk][w + 8 * u] * xv;
            }
        }
#pragma unroll
        for (int u = 0; u < 4; u++) S.Wm[w + 8 * u][lane] = acc[u];
        __syncthreads();
        // Y = T_b^T W
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int i = w + 8 * u;
            T y = T(0);
            if (i < bw)
                for (int j = 0; j <= i; j++) y += Tm[(i0 + j) + (size_t)(i0 + i) * ld] * S.Wm[j][lane];
            S.Ym[i][lane] = y;
        }
        // X[r][l] -= sum_i v_i[r] Y[i][l], chunk by chunk
        for (int rb = i0; rb < rows; rb += PW_KC) {
            __syncthreads();
            stage(rb, i0, bw);
            __syncthreads();
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int kk = w + 8 * u;
                T s2 = T(0);
                for (int ii = 0; ii < bw; ii++) s2 += S.vt[kk][ii] * S.Ym[ii][lane];
                S.xs[kk][lane] -= s2;
            }
            __syncthreads();
            for (int idx = tid; idx < PW_KC * PW_QB; idx += nth) {
                const int rr = rfast ? idx % PW_KC : idx / PW_QB, l = rfast ? idx / PW_KC : idx % PW_QB;
                const int r2 = rb + rr;
                if (l < nv && r2 < rows) base[r2 * sr + l * sv] = S.xs[rr][l];
            }
        }
    }
    __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(PV_THREADS) preserve_apply_kernel(Ctx<T> c, PhiCtx<T> P,
                                                                    const DSpars* __restrict__ items,
                                                                    const DAsn* __restrict__ pieces,
                                                                    const T* __restrict__ vstore,
                                                                    const T* __restrict__ tstore,
                                                                    const int* __restrict__ rank) {
    __shared__ WyTile<T> S;
    if (c.status->not_spd) return;
    const DSpars it = items[blockIdx.x];
    const int cl = it.cluster;
    const int rows = c.rows0[cl];
    const int k = rank[cl];
    if (k >= rows) return;
    if (blockIdx.y == 0 && threadIdx.x == 0) c.csize[cl] = k;
    const int ld = c.cap[cl];
    // the tile: 32-vector capacity tiles of the pieces, then those of phi
    int t = blockIdx.y, p = 0;
    for (; p < it.count; p++) {
        const int nt = (c.cap[pieces[it.first + p].nbr] + PW_QB - 1) / PW_QB;
        if (t < nt) break;
        t -= nt;
    }
    const int j0 = PW_QB * t;
    T* base;
    long long sr, sv;
    int nv;
    if (p < it.count) {
        const DAsn pc = pieces[it.first + p];
        const int n = c.csize[pc.nbr];
        if (j0 >= n) return;
        nv = min(PW_QB, n - j0);
        T* B = bptr(c, pc.block);
        const long long bld = c.blk[pc.block].ld;
        if (!pc.transposed) {
            base = B + (size_t)j0 * bld;
            sr = 1;
            sv = bld;
        } else {
            base = B + j0;
            sr = bld;
            sv = 1;
        }
    } else {
        if (j0 >= P.nphi) return;
        nv = min(PW_QB, P.nphi - j0);
        base = P.phis + P.off[cl] + (size_t)j0 * ld;
        sr = 1;
        sv = ld;
    }
    wy_qt_tile(vstore + it.v_off, tstore + it.v_off, ld, rows, k, base, sr, sv, nv, S);
}

// LoRaSp split (tree.cpp:1018-1064, keep_sibling): Q^T on a 32-vector tile of an original
// edge block, whose rows k .. rows-1 then go to the sibling's block (sibling x neighbour);
// the sibling's size becomes rows - k.  Grid (items, tiles over the original edges).
template <typename T>
__global__ void __launch_bounds__(PV_THREADS) lorasp_split_kernel(Ctx<T> c, const DSpars* __restrict__ items,
                                                                  const int* __restrict__ sibs,
                                                                  const int2* __restrict__ ranges,
                                                                  const int4* __restrict__ splits,
                                                                  const T* __restrict__ vstore,
                                                                  const T* __restrict__ tstore,
                                                                  const int* __restrict__ rank) {
    __shared__ WyTile<T> S;
    if (c.status->not_spd) return;
    const DSpars it = items[blockIdx.x];
    const int cl = it.cluster, sib = sibs[blockIdx.x];
    const int rows = c.rows0[cl];
    const int k = min(rank[cl], rows);
    if (blockIdx.y == 0 && threadIdx.x == 0) c.csize[sib] = c.rows0[sib] = rows - k;
    if (k >= rows) return;
    const int2 rg = ranges[blockIdx.x];
    int t = blockIdx.y, p = 0;
    for (; p < rg.y; p++) {
        const int nt = (c.cap[splits[rg.x + p].y] + PW_QB - 1) / PW_QB;
        if (t < nt) break;
        t -= nt;
    }
    if (p >= rg.y) return;
    const int4 sp = splits[rg.x + p];  // block, nbr, transposed, sibling block
    const int n = c.csize[sp.y];
    const int j0 = PW_QB * t;
    if (j0 >= n) return;
    const int nv = min(PW_QB, n - j0);
    T* B = bptr(c, sp.x);
    const long long bld = c.blk[sp.x].ld;
    T* base = sp.z ? B + j0 : B + (size_t)j0 * bld;
    const long long sr = sp.z ? bld : 1, sv = sp.z ? 1 : bld;
    const int ld = c.cap[cl];
    wy_qt_tile(vstore + it.v_off, tstore + it.v_off, ld, rows, k, base, sr, sv, nv, S);
    T* D = bptr(c, sp.w);
    const long long dld = c.blk[sp.w].ld;
    for (int idx = threadIdx.x; idx < (rows - k) * nv; idx += blockDim.x) {
        const int i = idx % (rows - k), l = idx / (rows - k);
        D[i + (size_t)(j0 + l) * dld] = base[(long long)(k + i) * sr + l * sv];
    }
}

int preserve_apply_tiles(const int* caps, int count, int nphi) {
    int t = (nphi + PW_QB - 1) / PW_QB;
    for (int p = 0; p < count; p++) t += (caps[p] + PW_QB - 1) / PW_QB;
    return std::max(1, t);
}

int lorasp_split_tiles(const int* caps, int count) {
    int t = 0;
    for (int p = 0; p < count; p++) t += (caps[p] + PW_QB - 1) / PW_QB;
    return std::max(1, t);
}

template <typename T>
void lorasp_split(Ctx<T> c, const DSpars* items, int n, int ytiles, const int* sibs, const int2* ranges,
                  const int4* splits, const T* vstore, const T* tstore, const int* rank, cudaStream_t s) {
    if (n == 0) return;
    lorasp_split_kernel<T><<<dim3((unsigned)n, (unsigned)ytiles), PV_THREADS, 0, s>>>(c, items, sibs, ranges, splits,
                                                                                     vstore, tstore, rank);
}

template <typename T>
void preserve_init(PhiCtx<T> P, const double* phinat, int n, const int* perm, const long long* dst, const int* ld,
                   cudaStream_t s) {
    const long long tot = (long long)n * P.nphi;
    if (tot == 0) return;
    phi_init_kernel<T><<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(P, phinat, n, perm, dst, ld);
}

template <typename T>
void preserve_scale(Ctx<T> c, PhiCtx<T> P, T* tmp, const int* clusters, const int* pivots, int count,
                    const int* perm_store, const long long* poff, cudaStream_t s) {
    if (count == 0) return;
    phi_scale_kernel<T><<<count, PV_THREADS, 0, s>>>(c, P, tmp, clusters, pivots, perm_store, poff);
}

template <typename T>
void preserve_merge(Ctx<T> c, PhiCtx<T> P, const int* parents, int np, const int* child_ptr, const int* child_idx,
                    const int* cpos, cudaStream_t s) {
    if (np == 0) return;
    phi_merge_kernel<T><<<np, PV_THREADS, 0, s>>>(c, P, parents, child_ptr, child_idx, cpos);
}

template <typename T>
void preserve_basis(Ctx<T> c, PhiCtx<T> P, const DSpars* items, int n, const DAsn* pieces, const T* signs,
                    const long long* soff, T* vstore, T* tauws, int* rank1, int* rank, bool adaptive, cudaStream_t s) {
    if (n == 0) return;
    preserve_basis_kernel<T><<<n, PV_THREADS, 0, s>>>(c, P, items, pieces, signs, soff, vstore, tauws, rank1, rank,
                                                      adaptive ? 1 : 0);
}

template <typename T>
void preserve_combine(Ctx<T> c, const DSpars* items, int n, const T* ws, T* vstore, T* tauws, const int* rank1,
                      int* rank, cudaStream_t s) {
    if (n == 0) return;
    preserve_combine_kernel<T><<<n, PV_THREADS, 0, s>>>(c, items, ws, vstore, tauws, rank1, rank);
}

template <typename T>
void preserve_apply(Ctx<T> c, PhiCtx<T> P, const DSpars* items, int n, int ytiles, const DAsn* pieces,
                    const T* vstore, const T* tstore, const int* rank, cudaStream_t s) {
    if (n == 0) return;
    preserve_apply_kernel<T><<<dim3((unsigned)n, (unsigned)ytiles), PV_THREADS, 0, s>>>(c, P, items, pieces, vstore,
                                                                                       tstore, rank);
}

#define SPAND_PRESERVE_INST(T)                                                                                     \
    template void preserve_init<T>(PhiCtx<T>, const double*, int, const int*, const long long*, const int*,         \
                                   cudaStream_t);                                                                  \
    template void preserve_scale<T>(Ctx<T>, PhiCtx<T>, T*, const int*, const int*, int, const int*,                 \
                                    const long long*, cudaStream_t);                                                \
    template void preserve_merge<T>(Ctx<T>, PhiCtx<T>, const int*, int, const int*, const int*, const int*,         \
                                    cudaStream_t);                                                                 \
    template void preserve_basis<T>(Ctx<T>, PhiCtx<T>, const DSpars*, int, const DAsn*, const T*,                   \
                                    const long long*, T*, T*, int*, int*, bool, cudaStream_t);                     \
    template void preserve_combine<T>(Ctx<T>, const DSpars*, int, const T*, T*, T*, const int*, int*, cudaStream_t); \
    template void preserve_apply<T>(Ctx<T>, PhiCtx<T>, const DSpars*, int, int, const DAsn*, const T*, const T*,    \
                                    const int*, cudaStream_t);                                                     \
    template void lorasp_split<T>(Ctx<T>, const DSpars*, int, int, const int*, const int2*, const int4*, const T*,  \
                                  const T*, const int*, cudaStream_t);

SPAND_PRESERVE_INST(float)
SPAND_PRESERVE_INST(double)

}  // namespace spand

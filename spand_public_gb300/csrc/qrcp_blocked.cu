// Blocked QRCP of the sparsification matrices: LAPACK's dlaqps panel scheme (Quintana-Orti,
// Sun and Bischof; LAWN 114) on the cluster-resident matrix of qrcp.cu.  The pivot
// sequence, the tie rule, the LAWN 176 norm downdating and the stop at
// |R_ii| / |R_00| < tol (choose_rank, src/util.cpp:434-452; the sparsification calls
// geqp3 from src/tree.cpp:1189-1224 and 1309) are those of the unblocked kernel; only
// the order of the floating-point updates differs.
//
// Why blocked: the unblocked kernel applies every reflector to the whole matrix at once
// (one dot and one rank-1 update per column: four shared-memory loads and one store per
// element per pivot step), which makes it shared-memory-bandwidth bound.  Here, inside a
// panel of up to QB_NB pivot steps, the trailing columns are only READ (one dot per
// column with the reflector held in registers); the reflectors' effect is accumulated in
// F (trailing column x panel step, dlaqps' F = tau A^T v corrected by the earlier
// reflectors) and applied once per panel as a rank-kb update with register tiles.  Per
// pivot step every CTA of the cluster:
//   1. picks the pivot from the entries every warp published (as qrcp.cu);
//   2. forms the pivot column u = a_p - V F_p^T from the owner's column and F row
//      (distributed shared memory) and its own copy of the panel's reflectors V, and
//      builds the Householder scalars itself (one block barrier for the norm);
//   3. computes F(:, k) = tau A^T v for its columns and the k dots V^T v (one block
//      barrier), corrects F(:, k) by them, updates row i of its columns, downdates the
//      norms and publishes; one cluster barrier;
//   4. at the end of a panel (QB_NB steps, a norm that must be recomputed, or the last
//      step) applies A -= V F^T below the panel's rows, recomputes the flagged norms and
//      publishes again; one more cluster barrier.
#include <cooperative_groups.h>

#include <climits>

#include "qrcp.cuh"

namespace spand {

namespace {

constexpr int QB_SLOTS = 16 * (QC_THREADS / 32);

template <typename T>
__device__ __forceinline__ T qb_warp_max(T v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ int qb_warp_min(int v) {
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ void qb_barrier(cooperative_groups::cluster_group& cl, int cs) {
    if (cs > 1) cl.sync();
    else __syncthreads();
}

}  // namespace

// RPL: rows per lane (matrices of up to 32 * RPL rows); a warp owns a column in the dots
// and in the panel update.  Shared memory per CTA (qb_need): the column slab (ld
// rows | 1), the panel reflectors V (ld rows | 1, QB_NB columns), F (QB_NB per slab
// column), the pivot column, the two partial-norm arrays, the permutation and the slab's
// column positions.  A matrix with more rows, or one whose slab does not fit, sets
// fallback[item] for the global-memory kernel.
template <typename T, int RPL>
__global__ void __launch_bounds__(QC_THREADS) qrcp_blocked_kernel(Ctx<T> c, const DSpars* __restrict__ items,
                                                                  const DAsn* __restrict__ pieces, T* ws, T* gslab,
                                                                  int* jpvt_ws, int* ipvt_ws, T* taus, int* rank_out,
                                                                  int* colcount, int* fallback, double tol,
                                                                  int smem_bytes, int vec_rows, QcProj<T> proj) {
    namespace cgx = cooperative_groups;
    (void)gslab;
    (void)vec_rows;
    (void)proj;
    cgx::cluster_group cl = cgx::this_cluster();
    const int CS = (int)cl.num_blocks();
    const int me = (int)cl.block_rank();
    const int item = blockIdx.x / CS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ T red[32];
    __shared__ T pubm[2][QB_SLOTS];  // per warp of the cluster: largest partial norm
    __shared__ int pubf[2][QB_SLOTS];  // first position inside its tie window
    __shared__ T pubn[2][QB_SLOTS];    // the partial norm at that position
    __shared__ int pubr[2][QB_SLOTS];  // a norm of the warp's columns must be recomputed
    __shared__ int pubx[2][QB_SLOTS];  // exact search with the global threshold
    __shared__ T s_alpha;
    if (c.status->not_spd) return;
    const DSpars it = items[item];
    const int rows = c.csize[it.cluster];
    int cols = 0;
    for (int p = 0; p < it.count; p++) cols += c.csize[pieces[it.first + p].nbr];
    const int mn = min(rows, cols);
    const int cpc = (cols + CS - 1) / CS;
    const int lda = rows | 1;
    const bool fits = rows <= 32 * RPL && qb_need(rows, cols, CS, (int)sizeof(T)) <= smem_bytes;
    if (threadIdx.x == 0 && me == 0) {
        fallback[item] = (mn > 0 && tol < 1.0 && !fits) ? 1 : 0;
        if (fallback[item]) atomicOr(&c.status->overflow, 1);
        colcount[item] = cols;
    }
    int* jpg = jpvt_ws + it.col_off;
    int* ipg = ipvt_ws + it.col_off;
    if (mn == 0 || tol >= 1.0) {
        // choose_rank gives 0 for an empty diagonal and for tol >= 1: no reflectors
        if (me == 0) {
            for (int j = threadIdx.x; j < cols; j += blockDim.x) {
                jpg[j] = j;
                ipg[j] = j;
            }
            if (threadIdx.x == 0) rank_out[it.cluster] = 0;
        }
        return;
    }
    if (!fits) return;
    const int c0 = me * cpc;
    T* A = reinterpret_cast<T*>(smem_raw);
    T* Vp = A + (size_t)lda * cpc;          // panel reflectors, column l at Vp + l * lda
    T* F = Vp + (size_t)lda * QB_NB;        // F(j, l) at F[j * QB_NB + l]
    T* vsh = F + (size_t)cpc * QB_NB;       // the pivot column u (unscaled reflector)
    T* auxv = vsh + rows;                   // -tau V^T v of the current step
    T* vn1 = auxv + QB_NB;
    T* vn2 = vn1 + cpc;
    int* perm = reinterpret_cast<int*>(vn2 + cpc);
    int* pos = perm + cols;
    const int c1 = min(cols, c0 + cpc);
    const int nloc = max(0, c1 - c0);
    const int tid = threadIdx.x, nth = blockDim.x;
    const int lane = tid & 31, w = tid >> 5, nw = nth >> 5;
    qc_gather_slab(c, it, pieces, rows, c0, c1, A, lda);
    for (int p = tid; p < cols; p += nth) perm[p] = p;
    for (int j = tid; j < nloc; j += nth) pos[j] = c0 + j;
    __syncthreads();
    for (int j = w; j < nloc; j += nw) {
        const T* a = A + (size_t)j * lda;
        T s = 0;
        for (int r = lane; r < rows; r += 32) s += a[r] * a[r];
        s = warp_sum(s);
        if (lane == 0) {
            vn1[j] = dsqrt(s);
            vn2[j] = vn1[j];
        }
    }
    const T tie = T(1) - qrcp_tie<T>();
    const T tol3z = dsqrt(sizeof(T) == 8 ? T(2.220446049250313e-16) : T(1.1920929e-07));
    const int E = CS * nw;
    const int slot = me * nw + w;
    // A warp publishes into every CTA: the largest partial norm m of its lanes' columns at
    // positions >= from, the first position inside m's tie window with its norm, and
    // whether one of its columns waits for a recomputed norm.  Lane columns: j = tid + q nth.
    auto publish = [&](int par, int from, T mlane, int flag) {
        const T m = qb_warp_max(mlane);
        const T thr = m * tie;
        int f = INT_MAX;
        T fn = 0;
        for (int j = tid; j < nloc; j += nth) {
            const int p = pos[j];
            if (p >= from && vn1[j] >= thr && p < f) {
                f = p;
                fn = vn1[j];
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const int of = __shfl_xor_sync(0xffffffffu, f, o);
            const T on = __shfl_xor_sync(0xffffffffu, fn, o);
            if (of < f) {
                f = of;
                fn = on;
            }
        }
        const int any = __any_sync(0xffffffffu, flag) ? 1 : 0;
        if (lane < CS) {
            *cl.map_shared_rank(&pubm[par][slot], lane) = m;
            *cl.map_shared_rank(&pubf[par][slot], lane) = f;
            *cl.map_shared_rank(&pubn[par][slot], lane) = fn;
            *cl.map_shared_rank(&pubr[par][slot], lane) = any;
        }
    };
    __syncthreads();  // norms of every slab column written
    int pc = 0;       // publications so far; the latest sits in buffer pc & 1
    {
        T m = 0;
        for (int j = tid; j < nloc; j += nth) m = fmax(m, vn1[j]);
        publish(0, 0, m, 0);
    }
    qb_barrier(cl, CS);
    int rank = mn;
    T r00 = 0;
    int pend = -1;  // local column awaiting its reflector (vsh rows > pend_i scaled by pend_sc, beta at pend_i)
    T pend_beta = 0, pend_sc = 0;
    int pend_i = 0;
    int i0 = 0;  // first pivot step of the current panel
    for (int i = 0; i < mn; i++) {
        const int par = pc & 1;
        const int k = i - i0;  // step inside the panel
        // (1) pivot from the published entries (the unblocked kernel's rule)
        T gmax = 0;
        for (int e = lane; e < E; e += 32) gmax = fmax(gmax, pubm[par][e]);
        gmax = qb_warp_max(gmax);
        const T thr = gmax * tie;
        int pvt = INT_MAX;
        bool amb = false;
        for (int e = lane; e < E; e += 32) {
            const T m = pubm[par][e];
            if (m >= thr) {
                if (pubn[par][e] >= thr) pvt = min(pvt, pubf[par][e]);
                else amb = true;
            }
        }
        pvt = qb_warp_min(pvt);
        if (__any_sync(0xffffffffu, amb)) {
            int f = INT_MAX;
            for (int j = tid; j < nloc; j += nth) {
                const int p = pos[j];
                if (p >= i && vn1[j] >= thr && p < f) f = p;
            }
            f = qb_warp_min(f);
            if (lane < CS) *cl.map_shared_rank(&pubx[par][slot], lane) = f;
            qb_barrier(cl, CS);
            pvt = INT_MAX;
            for (int e = lane; e < E; e += 32) pvt = min(pvt, pubx[par][e]);
            pvt = qb_warp_min(pvt);
        }
        if (pvt < i || pvt >= cols) pvt = i;  // all norms NaN: keep the current position
        const int phys = perm[pvt];
        const int phys_i = perm[i];
        const int own = phys / cpc, lj = phys - own * cpc;
        // (2) u = a_p - V F_p^T on rows >= i (the owner's column and F row), into vsh; the
        // previous reflector into its column (owner), with the same row -> thread map
        const T* src = (own == me ? A : cl.map_shared_rank(A, own)) + (size_t)lj * lda;
        const T* fsrc = (own == me ? F : cl.map_shared_rank(F, own)) + (size_t)lj * QB_NB;
        T fp[QB_NB];
#pragma unroll
        for (int l = 0; l < QB_NB; l++) fp[l] = l < k ? fsrc[l] : T(0);
        T* apend = pend >= 0 ? A + (size_t)pend * lda : nullptr;
        T part = 0;
        for (int r = tid; r < rows; r += nth) {
            if (apend && r > pend_i) apend[r] = vsh[r] * pend_sc;
            if (r >= i) {
                T u = src[r];
#pragma unroll
                for (int l = 0; l < QB_NB; l++)
                    if (l < k) u -= Vp[r + (size_t)l * lda] * fp[l];
                vsh[r] = u;
                if (r == i) s_alpha = u;
                else part += u * u;
            }
        }
        if (apend && tid == 0) apend[pend_i] = pend_beta;
        pend = -1;
        part = warp_sum(part);
        if (lane == 0) red[w] = part;
        __syncthreads();  // vsh, partial norms, alpha; every thread has read perm
        T xnorm2 = 0;
        for (int q = 0; q < nw; q++) xnorm2 += red[q];
        const T alpha = s_alpha;
        const T xnorm = dsqrt(xnorm2);
        T beta, tu, sc;
        if (xnorm == T(0)) {
            beta = alpha;
            tu = 0;
            sc = 0;
        } else {
            // -sign(alpha) |(alpha, x)| with sign(-0) = +1 (the oracle's rule)
            beta = alpha >= T(0) ? -hypot(alpha, xnorm) : hypot(alpha, xnorm);
            tu = (beta - alpha) / beta;
            sc = T(1) / (alpha - beta);
        }
        const T rii = fabs(beta);
        if (i == 0) r00 = rii;
        if (tol != 0.0 && i >= 1 && !(rii / r00 >= T(tol))) {
            rank = i;
            break;
        }
        if (me == 0 && tid == 0) taus[it.tau_off + i] = tu;
        if (tid == 0) {
            perm[i] = phys;
            perm[pvt] = phys_i;
        }
        // (3) the reflector v = [1; sc u(i+1:)] in registers (lane rows r = lane + 32 t) and in
        // V(:, k); the dots F(j, k) = tau a_j^T v of this CTA's trailing columns and the
        // k dots V(:, l)^T v, a warp per column
        T v[RPL];
#pragma unroll
        for (int t = 0; t < RPL; t++) {
            const int r = lane + 32 * t;
            v[t] = (r < rows && r >= i) ? (r == i ? T(1) : sc * vsh[r]) : T(0);
        }
        for (int r = tid; r < rows; r += nth)
            if (r >= i) Vp[r + (size_t)k * lda] = r == i ? T(1) : sc * vsh[r];
        for (int q = w; q < k + nloc; q += nw) {
            const T* col;
            if (q < k) {
                col = Vp + (size_t)q * lda;
            } else {
                const int j = q - k;
                if (c0 + j == phys || pos[j] < i) continue;  // pivoted (warp-uniform)
                col = A + (size_t)j * lda;
            }
            T s = 0;
#pragma unroll
            for (int t = 0; t < RPL; t++) {
                const int r = lane + 32 * t;
                if (r >= i && r < rows) s += col[r] * v[t];
            }
            s = warp_sum(s);
            if (lane == 0) {
                if (q < k) auxv[q] = -tu * s;
                else F[(size_t)(q - k) * QB_NB + k] = tu * s;
            }
        }
        __syncthreads();  // auxv, F(:, k) and V(:, k) visible
        // (4) per trailing column (a thread each): F(j, k) += F(j, 0:k) auxv, row i updated
        // by the panel's reflectors, norm downdated (LAWN 176); a norm that must be
        // recomputed is flagged by vn2 < 0 and ends the panel
        T mloc = 0;
        int flag = 0;
        for (int j = tid; j < nloc; j += nth) {
            const int ph = c0 + j;
            if (ph != phys && pos[j] >= i) {
                T* Fj = F + (size_t)j * QB_NB;
                T f = Fj[k];
                for (int l = 0; l < k; l++) f += Fj[l] * auxv[l];
                Fj[k] = f;
                T* aij = A + i + (size_t)j * lda;
                T a = *aij;
                for (int l = 0; l < k; l++) a -= Vp[i + (size_t)l * lda] * Fj[l];
                a -= f;
                *aij = a;
                const T v1 = vn1[j];
                T newv = v1;
                if (v1 != T(0)) {
                    T temp = fabs(a) / v1;
                    temp = T(1) - temp * temp;
                    temp = temp > T(0) ? temp : T(0);
                    const T rr = v1 / vn2[j];
                    if (temp * rr * rr <= tol3z) {
                        vn2[j] = T(-1);
                        flag = 1;
                    } else {
                        newv = v1 * dsqrt(temp);
                    }
                }
                vn1[j] = newv;
                if (ph == phys_i) pos[j] = pvt;
                mloc = fmax(mloc, newv);
            }
            if (ph == phys) pos[j] = i;
        }
        if (own == me) {
            pend = lj;
            pend_i = i;
            pend_beta = beta;
            pend_sc = sc;
        }
        if (i + 1 == mn) break;
        publish(par ^ 1, i + 1, mloc, flag);
        pc++;
        qb_barrier(cl, CS);
        bool panel_end = k + 1 == QB_NB;
        {
            int any = 0;
            for (int e = lane; e < E; e += 32) any |= pubr[pc & 1][e];
            panel_end |= __any_sync(0xffffffffu, any) != 0;
        }
        if (!panel_end) continue;
        // (5) panel end: A(i+1:, j) -= V(i+1:, 0:k+1) F(j, 0:k+1)^T for the trailing columns,
        // flagged norms recomputed from the updated columns, then published again
        const int kb = k + 1;
        for (int j = w; j < nloc; j += nw) {
            if (pos[j] <= i) continue;  // pivoted (warp-uniform)
            T* a = A + (size_t)j * lda;
            const T* Fj = F + (size_t)j * QB_NB;
            T acc[RPL];
#pragma unroll
            for (int t = 0; t < RPL; t++) {
                const int r = lane + 32 * t;
                acc[t] = (r > i && r < rows) ? a[r] : T(0);
            }
            for (int l = 0; l < kb; l++) {
                const T fl = Fj[l];
                const T* Vl = Vp + (size_t)l * lda;
#pragma unroll
                for (int t = 0; t < RPL; t++) {
                    const int r = lane + 32 * t;
                    if (r > i && r < rows) acc[t] -= Vl[r] * fl;
                }
            }
            T q2 = 0;
#pragma unroll
            for (int t = 0; t < RPL; t++) {
                const int r = lane + 32 * t;
                if (r > i && r < rows) {
                    a[r] = acc[t];
                    q2 += acc[t] * acc[t];
                }
            }
            if (vn2[j] < T(0)) {
                q2 = warp_sum(q2);
                if (lane == 0) {
                    const T nv = (i < rows - 1) ? dsqrt(q2) : T(0);
                    vn1[j] = nv;
                    vn2[j] = nv;
                }
            }
        }
        __syncthreads();
        {
            T m = 0;
            for (int j = tid; j < nloc; j += nth)
                if (pos[j] > i) m = fmax(m, vn1[j]);
            publish((pc + 1) & 1, i + 1, m, 0);
        }
        pc++;
        qb_barrier(cl, CS);
        i0 = i + 1;
    }
    // no CTA reads another's shared memory after this barrier (nor leaves before it)
    qb_barrier(cl, CS);
    if (pend >= 0) {
        T* a = A + (size_t)pend * lda;
        for (int r = pend_i + 1 + tid; r < rows; r += nth) a[r] = vsh[r] * pend_sc;
        if (tid == 0) a[pend_i] = pend_beta;
    }
    __syncthreads();
    const int ld = c.cap[it.cluster];
    T* W = ws + it.ws_off;
    for (int j = w; j < nloc; j += nw) {
        const int p = pos[j];
        const T* a = A + (size_t)j * lda;
        T* dst = W + (size_t)p * ld;
        for (int r = lane; r < rows; r += 32) dst[r] = a[r];
        if (lane == 0) {
            jpg[p] = c0 + j;
            ipg[c0 + j] = p;
        }
    }
    if (me == 0 && tid == 0) rank_out[it.cluster] = rank;
}

template <typename T>
QcKernel<T> qrcp_blocked_kernel_ptr(int rpl) {
    switch (rpl) {
        case 1: return qrcp_blocked_kernel<T, 1>;
        case 2: return qrcp_blocked_kernel<T, 2>;
        case 4: return qrcp_blocked_kernel<T, 4>;
        case 8: return qrcp_blocked_kernel<T, 8>;
        case 12: return qrcp_blocked_kernel<T, 12>;
        default: return nullptr;
    }
}

template QcKernel<float> qrcp_blocked_kernel_ptr<float>(int);
template QcKernel<double> qrcp_blocked_kernel_ptr<double>(int);

}  // namespace spand

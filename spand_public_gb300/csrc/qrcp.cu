// QRCP of the sparsification matrices: LAPACK dgeqp3/dlaqp2 (Householder QR with
// column pivoting, LAWN 176 norm downdating) stopped as soon as |R_ii| / |R_00| < tol
// (choose_rank, src/util.cpp:434-452; the sparsification calls it from
// src/tree.cpp:1189-1224).  The pivot is the first column whose partial norm lies within
// a relative qrcp_tie<T>() of the largest (the oracle's rule).
#include <cooperative_groups.h>

#include <climits>

#include "qrcp.cuh"

namespace spand {

// QRCP without column movement.  The sparsification matrix stays in the shared memory of
// a thread-block cluster (CS CTAs, column slabs); a column never moves: the pivoting is
// tracked as a permutation (perm: position -> column, replicated in every CTA; pos:
// column -> position for the slab's own columns).  G threads per column.  Per pivot step i:
//   1. every warp reads the entries published by every warp of the cluster (largest
//      partial norm m of its columns, first position inside the tie window of m) and
//      derives the pivot with shuffles; exact as long as no warp maximum lies inside the
//      tie window below the global one (else every warp searches with the global
//      threshold, one more barrier);
//   2. the owner writes the previous reflector into its column and every CTA reads the
//      pivot column (distributed shared memory) with the same row -> thread map, so
//      neither needs a barrier; one barrier for the column norm, then every thread forms
//      the Householder scalars itself;
//   3. every CTA applies H = I - tau v v^T, v = [1; sc * x] (the unscaled column x stays
//      in shared memory, sc is folded into the update), downdates the norms (LAWN 176),
//      and every warp publishes its next entry into every CTA; one cluster barrier.
// At the end the slabs are written to the global workspace in LAPACK's column order
// (position p holds column perm[p]).

template <typename T>
__device__ __forceinline__ T warp_max(T v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ int warp_min(int v) {
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ void qc_barrier(cooperative_groups::cluster_group& cl, int cs) {
    if (cs > 1) cl.sync();
    else __syncthreads();
}

// GS = false: the column slabs live in the CTAs' shared memory; a matrix that does not fit
// sets fallback[item].  GS = true: the same algorithm with the slabs in global memory (the
// second workspace gslab, L2-resident), for exactly the matrices flagged by the
// shared-memory launch; the CTAs read other slabs' columns with L2-only loads.
// the vectorised trailing update needs at least this many rows (two vectors per lane)
constexpr int QC_VEC_ROWS = 64;

// sixteen bytes of a column, loaded and stored as one shared-memory vector
template <typename T>
struct alignas(16) QcPack {
    T e[16 / sizeof(T)];
};

// NT: the largest CTA this instantiation is launched with (QC_THREADS, or QC_WIDE_THREADS
// for the waves whose shared memory admits one CTA per SM: twice the warps on each slab)
template <typename T, bool GS, int NT>
__global__ void __launch_bounds__(NT) qrcp_cluster_kernel(Ctx<T> c, const DSpars* __restrict__ items,
                                                                  const DAsn* __restrict__ pieces, T* ws, T* gslab,
                                                                  int* jpvt_ws, int* ipvt_ws, T* taus,
                                                                  int* rank_out, int* colcount, int* fallback,
                                                                  double tol, int smem_bytes, int vec_rows,
                                                                  QcProj<T> proj) {
    pdl_wait_and_release();
    namespace cgx = cooperative_groups;
    cgx::cluster_group cl = cgx::this_cluster();
    const int CS = (int)cl.num_blocks();
    const int me = (int)cl.block_rank();
    const int item = blockIdx.x / CS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int QC_SLOTS = 16 * (NT / 32);  // warps of the largest cluster
    __shared__ T red[32];
    __shared__ T pubm[2][QC_SLOTS];  // per warp of the cluster: largest partial norm
    __shared__ int pubf[2][QC_SLOTS];  // first position inside its tie window
    __shared__ T pubn[2][QC_SLOTS];    // the partial norm at that position
    __shared__ int pubx[2][QC_SLOTS];  // exact search with the global threshold
    __shared__ T s_alpha;
    if (c.status->not_spd) return;
    if (GS && !fallback[item]) return;  // handled by the shared-memory launch
    const DSpars it = items[item];
    const int rows = c.csize[it.cluster];
    int cols = 0;
    for (int p = 0; p < it.count; p++) cols += c.csize[pieces[it.first + p].nbr];
    const int mn = min(rows, cols);
    const int cpc = (cols + CS - 1) / CS;
    // the vectorised update (16-byte shared-memory vectors, eight lanes per column) for
    // slabs of at least vec_rows rows; the scalar update (odd leading dimension) below
    constexpr int VW = 16 / (int)sizeof(T);
    const bool vec = !GS && rows >= max(vec_rows, QC_VEC_ROWS);
    const int lda = GS ? c.cap[it.cluster] : (vec ? (rows + VW - 1) / VW * VW : (rows | 1));
    const bool fits = GS ? qc_small_need(rows, cols, CS, (int)sizeof(T)) <= smem_bytes
                         : qc_need(rows, cols, CS, (int)sizeof(T)) <= smem_bytes;
    const int r1 = proj.q ? proj.rank1[it.cluster] : 0;
    const bool spanned = proj.q && r1 >= rows;
    if (!GS && threadIdx.x == 0 && me == 0) {
        fallback[item] = (mn > 0 && tol < 1.0 && !fits && !spanned) ? 1 : 0;
        if (fallback[item]) atomicOr(&c.status->overflow, 1);
        colcount[item] = cols;
    }
    int* jpg = jpvt_ws + it.col_off;
    int* ipg = ipvt_ws + it.col_off;
    if (mn == 0 || tol >= 1.0 || spanned) {
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
    T* Aitem = gslab + it.ws_off;  // GS: the whole matrix, column j at Aitem + j * lda
    T* A = GS ? Aitem + (size_t)c0 * lda : reinterpret_cast<T*>(smem_raw);
    T* vsh = GS ? reinterpret_cast<T*>(smem_raw) : A + (size_t)lda * cpc;
    T* vn1 = vsh + (GS ? rows : lda);
    T* vn2 = vn1 + cpc;
    int* perm = reinterpret_cast<int*>(vn2 + cpc);
    int* pos = perm + cols;
    const int c1 = min(cols, c0 + cpc);
    const int nloc = max(0, c1 - c0);
    const int tid = threadIdx.x, nth = blockDim.x;
    const int lane = tid & 31, w = tid >> 5, nw = nth >> 5;
    // gather the slab of Asn = [A_sn | A_ns^T]
    qc_gather_slab(c, it, pieces, rows, c0, c1, A, lda);
    if (vec) {
        // the vectors' padding rows stay zero in every column and in the reflector
        const int pad = lda - rows;
        for (int idx = tid; idx < pad * nloc; idx += nth) A[rows + idx % pad + (size_t)(idx / pad) * lda] = T(0);
        for (int r = rows + tid; r < lda; r += nth) vsh[r] = T(0);
    }
    for (int p = tid; p < cols; p += nth) perm[p] = p;
    for (int j = tid; j < nloc; j += nth) pos[j] = c0 + j;
    __syncthreads();
    if (r1 > 0) {
        // a <- (I - Q1 Q1^T) a, one basis vector at a time, by the warp that owns column a
        const T* Q1 = proj.q + it.v_off;
        const int ldq = c.cap[it.cluster];
        for (int j = w; j < nloc; j += nw) {
            T* a = A + (size_t)j * lda;
            for (int k = 0; k < r1; k++) {
                const T* q = Q1 + (size_t)k * ldq;
                T s = 0;
                for (int r = lane; r < rows; r += 32) s += q[r] * a[r];
                s = warp_sum(s);
                for (int r = lane; r < rows; r += 32) a[r] -= s * q[r];
            }
        }
        __syncwarp();
    }
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
    // threads per column for the trailing update
    int G = 1;
    while (G < 8 && (nloc * G * 2 <= nth || rows >= 64 * G)) G *= 2;
    if (vec) {
        // eight lanes per column, or four where that takes the slab's columns in fewer
        // rounds (the same vectors per lane, one fixed round cost less)
        const int g8 = nth / 8, g4 = nth / 4;
        G = (nloc + g4 - 1) / g4 < (nloc + g8 - 1) / g8 ? 4 : 8;
    }
    const int gid = tid / G, gl = tid % G, ngroups = nth / G;
    const T tie = T(1) - qrcp_tie<T>();
    const T tol3z = dsqrt(sizeof(T) == 8 ? T(2.220446049250313e-16) : T(1.1920929e-07));

    const int E = CS * nw;          // published entries: every warp of every CTA
    const int slot = me * nw + w;   // this warp's entry
    // A warp publishes into every CTA (largest partial norm m of its columns at positions
    // >= from, first position inside the tie window of m).  mlane: the lane's maximum over
    // its column group's columns (0 if it leads no group).
    auto publish = [&](int par, int from, T mlane) {
        const T m = warp_max(mlane);
        const T thr = m * tie;
        int f = INT_MAX;
        T fn = 0;
        if (gl == 0)
            for (int j = gid; j < nloc; j += ngroups) {
                const int p = pos[j];
                if (p >= from && vn1[j] >= thr && p < f) {
                    f = p;
                    fn = vn1[j];
                }
            }
        // first position with its norm (the norm rides along the minimum)
        for (int o = 16; o > 0; o >>= 1) {
            const int of = __shfl_xor_sync(0xffffffffu, f, o);
            const T on = __shfl_xor_sync(0xffffffffu, fn, o);
            if (of < f) {
                f = of;
                fn = on;
            }
        }
        if (lane < CS) {
            *cl.map_shared_rank(&pubm[par][slot], lane) = m;
            *cl.map_shared_rank(&pubf[par][slot], lane) = f;
            *cl.map_shared_rank(&pubn[par][slot], lane) = fn;
        }
    };

    __syncthreads();  // norms of every slab column written
    {
        T m = 0;
        if (gl == 0)
            for (int j = gid; j < nloc; j += ngroups) m = fmax(m, vn1[j]);
        publish(0, 0, m);
    }
    qc_barrier(cl, CS);
    int rank = mn;
    T r00 = 0;
    int pend = -1;  // local column awaiting its reflector (scaled vsh rows > pend_i, beta at pend_i)
    T pend_beta = 0, pend_sc = 0;
    int pend_i = 0;
    for (int i = 0; i < mn; i++) {
        const int par = i & 1;
        // (1) pivot, in every warp from the published entries
        // (the entry loops unrolled over the slot bound: their loads issue together)
        T gmax = 0;
#pragma unroll
        for (int q = 0; q < QC_SLOTS / 32; q++) {
            const int e = lane + 32 * q;
            if (e < E) gmax = fmax(gmax, pubm[par][e]);
        }
        gmax = warp_max(gmax);
        const T thr = gmax * tie;
        int pvt = INT_MAX;
        bool amb = false;
        // a warp whose maximum reaches the global window published the first position of
        // its own (wider or equal) window; where that column also reaches the global
        // threshold it is the warp's first candidate, else the warp must search again
#pragma unroll
        for (int q = 0; q < QC_SLOTS / 32; q++) {
            const int e = lane + 32 * q;
            if (e < E) {
                const T m = pubm[par][e];
                const T fnm = pubn[par][e];
                const int fpos = pubf[par][e];
                if (m >= thr) {
                    if (fnm >= thr) pvt = min(pvt, fpos);
                    else amb = true;
                }
            }
        }
        pvt = warp_min(pvt);
        if (__any_sync(0xffffffffu, amb)) {
            // a warp maximum inside the tie window below the global one: every warp searches
            // its columns with the global threshold (the same decision in every warp)
            int f = INT_MAX;
            if (gl == 0)
                for (int j = gid; j < nloc; j += ngroups) {
                    const int p = pos[j];
                    if (p >= i && vn1[j] >= thr && p < f) f = p;
                }
            f = warp_min(f);
            if (lane < CS) *cl.map_shared_rank(&pubx[par][slot], lane) = f;
            qc_barrier(cl, CS);
            pvt = INT_MAX;
            for (int e = lane; e < E; e += 32) pvt = min(pvt, pubx[par][e]);
            pvt = warp_min(pvt);
        }
        if (pvt < i || pvt >= cols) pvt = i;  // all norms NaN: keep the current position
        const int phys = perm[pvt];
        const int phys_i = perm[i];
        const int own = phys / cpc, lj = phys - own * cpc;
        // (2) the previous reflector into its column (owner) and the pivot column into vsh,
        // both with the row -> thread map r = tid (mod nth): a thread reads its old vsh rows
        // before it overwrites them
        const T* src = GS ? Aitem + (size_t)phys * lda
                          : (own == me ? A : cl.map_shared_rank(A, own)) + (size_t)lj * lda;
        T* apend = pend >= 0 ? A + (size_t)pend * lda : nullptr;
        T part = 0;
        // vsh holds zeros from the start of row i's 16-byte vector through row i, so that the
        // vectorised update can run over whole vectors (row i itself is updated apart)
        const int rv = (i + 1) & ~(VW - 1);
        for (int r = tid; r < rows; r += nth) {
            if (apend && r > pend_i) apend[r] = vsh[r] * pend_sc;
            if (r >= i) {
                const T v = GS ? __ldcg(src + r) : src[r];
                vsh[r] = r == i ? T(0) : v;
                if (r == i) s_alpha = v;
                else part += v * v;
            } else if (r >= rv) {
                vsh[r] = T(0);
            }
        }
        if (apend && tid == 0) apend[pend_i] = pend_beta;
        pend = -1;
        part = warp_sum(part);
        if (lane == 0) red[w] = part;
        __syncthreads();  // partial norms, alpha; every thread has read perm
        const T xnorm2 = warp_sum(lane < nw ? red[lane] : T(0));
        const T alpha = s_alpha;
        const T xnorm = dsqrt(xnorm2);
        T beta, tu, sc;
        if (xnorm == T(0)) {
            beta = alpha;
            tu = 0;
            sc = 0;
        } else {
            // -sign(alpha) |(alpha, x)| with sign(-0) = +1 (the oracle's rule: a zero leading
            // entry counts as positive whatever sign bit rounding left on it)
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
        // (3) H = I - tu v v^T, v = [1; sc * vsh[i+1:]], on this slab's columns at positions
        // >= i (positions after the swap), norms downdated (LAWN 176) by the group's first
        // lane.  The loop runs the same number of times in every thread so that the group
        // shuffles always see all 32 lanes.
        T mloc = 0;
        for (int base = 0; base < nloc; base += ngroups) {
            const int j = base + gid;
            const int ph = c0 + j;
            const bool active = j < nloc && ph != phys && pos[j] >= i;
            T* aj = A + (size_t)(active ? j : 0) * lda;
            T s = 0;
            if (vec) {
                if (active && tu != T(0)) {
                    T s0 = 0, s1 = 0;
                    for (int r = rv + VW * gl; r < rows; r += VW * G) {
                        const QcPack<T> a = *reinterpret_cast<const QcPack<T>*>(aj + r);
                        const QcPack<T> v = *reinterpret_cast<const QcPack<T>*>(vsh + r);
#pragma unroll
                        for (int e = 0; e < VW; e += 2) {
                            s0 += v.e[e] * a.e[e];
                            s1 += v.e[e + 1] * a.e[e + 1];
                        }
                    }
                    s = s0 + s1;
                }
            } else if (active && tu != T(0)) {
                T s0 = 0, s1 = 0, s2 = 0, s3 = 0;
                int r = i + 1 + gl;
                for (; r + 3 * G < rows; r += 4 * G) {
                    s0 += vsh[r] * aj[r];
                    s1 += vsh[r + G] * aj[r + G];
                    s2 += vsh[r + 2 * G] * aj[r + 2 * G];
                    s3 += vsh[r + 3 * G] * aj[r + 3 * G];
                }
                for (; r < rows; r += G) s0 += vsh[r] * aj[r];
                s = (s0 + s1) + (s2 + s3);
            }
            for (int o = G >> 1; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            const T ai0 = __shfl_sync(0xffffffffu, (active && gl == 0) ? aj[i] : T(0), (lane / G) * G);
            if (vec && active && tu != T(0)) {
                const T coef = tu * (ai0 + sc * s);
                const T cr = coef * sc;
                for (int r = rv + VW * gl; r < rows; r += VW * G) {
                    QcPack<T> a = *reinterpret_cast<const QcPack<T>*>(aj + r);
                    const QcPack<T> v = *reinterpret_cast<const QcPack<T>*>(vsh + r);
#pragma unroll
                    for (int e = 0; e < VW; e++) a.e[e] -= cr * v.e[e];
                    *reinterpret_cast<QcPack<T>*>(aj + r) = a;
                }
                // after the vectors: the one holding row i (this lane's first) rewrote it unchanged
                if (gl == 0) aj[i] = ai0 - coef;
            } else if (active && tu != T(0)) {
                const T coef = tu * (ai0 + sc * s);
                const T cr = coef * sc;
                if (gl == 0) aj[i] = ai0 - coef;
                int r = i + 1 + gl;
                for (; r + 3 * G < rows; r += 4 * G) {
                    const T a0 = aj[r], a1 = aj[r + G], a2 = aj[r + 2 * G], a3 = aj[r + 3 * G];
                    aj[r] = a0 - cr * vsh[r];
                    aj[r + G] = a1 - cr * vsh[r + G];
                    aj[r + 2 * G] = a2 - cr * vsh[r + 2 * G];
                    aj[r + 3 * G] = a3 - cr * vsh[r + 3 * G];
                }
                for (; r < rows; r += G) aj[r] -= cr * vsh[r];
            }
            __syncwarp();
            int recompute = 0;
            T newv = 0;
            if (active && gl == 0) {
                const T v1 = vn1[j];
                newv = v1;
                if (v1 != T(0)) {
                    T temp = fabs(aj[i]) / v1;
                    temp = T(1) - temp * temp;
                    temp = temp > T(0) ? temp : T(0);
                    const T rr = v1 / vn2[j];
                    if (temp * rr * rr <= tol3z) recompute = 1;
                    else newv = v1 * dsqrt(temp);
                }
            }
            recompute = __shfl_sync(0xffffffffu, recompute, (lane / G) * G);
            T q2 = 0;
            if (active && recompute) {
                T q0 = 0, q1 = 0, q2b = 0, q3 = 0;
                int r = i + 1 + gl;
                for (; r + 3 * G < rows; r += 4 * G) {
                    q0 += aj[r] * aj[r];
                    q1 += aj[r + G] * aj[r + G];
                    q2b += aj[r + 2 * G] * aj[r + 2 * G];
                    q3 += aj[r + 3 * G] * aj[r + 3 * G];
                }
                for (; r < rows; r += G) q0 += aj[r] * aj[r];
                q2 = (q0 + q1) + (q2b + q3);
            }
            for (int o = G >> 1; o > 0; o >>= 1) q2 += __shfl_xor_sync(0xffffffffu, q2, o);
            if (active && gl == 0) {
                if (recompute) {
                    newv = (i < rows - 1) ? dsqrt(q2) : T(0);
                    vn2[j] = newv;
                }
                vn1[j] = newv;
                if (ph == phys_i) pos[j] = pvt;
                mloc = fmax(mloc, newv);
            }
            if (j < nloc && gl == 0 && ph == phys) pos[j] = i;
        }
        if (own == me) {
            pend = lj;
            pend_i = i;
            pend_beta = beta;
            pend_sc = sc;
        }
        if (i + 1 < mn) {
            publish(par ^ 1, i + 1, mloc);
            qc_barrier(cl, CS);
        }
    }
    // no CTA reads another's shared memory after this barrier (nor leaves before it)
    qc_barrier(cl, CS);
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
QcKernel<T> qrcp_smem_kernel_ptr(int threads) {
    if (threads > QC_THREADS) return qrcp_cluster_kernel<T, false, QC_WIDE_THREADS>;
    return qrcp_cluster_kernel<T, false, QC_THREADS>;
}

template <typename T>
QcKernel<T> qrcp_gslab_kernel_ptr() {
    return qrcp_cluster_kernel<T, true, QC_THREADS>;
}

template QcKernel<float> qrcp_smem_kernel_ptr<float>(int);
template QcKernel<double> qrcp_smem_kernel_ptr<double>(int);
template QcKernel<float> qrcp_gslab_kernel_ptr<float>();
template QcKernel<double> qrcp_gslab_kernel_ptr<double>();

}  // namespace spand

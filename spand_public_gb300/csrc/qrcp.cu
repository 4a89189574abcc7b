// QRCP of the sparsification matrices: LAPACK dgeqp3/dlaqp2 (Householder QR with
// column pivoting, LAWN 176 norm downdating) stopped as soon as |R_ii| / |R_00| < tol
// (choose_rank, src/util.cpp:434-452; the sparsification calls it from
// src/tree.cpp:1189-1224).  The pivot is the first column whose partial norm lies within
// a relative qrcp_tie<T>() of the largest (the oracle's rule).
#include <cooperative_groups.h>

#include <climits>

#include "qrcp.cuh"

namespace spand {

// QRCP, version without column movement.  The sparsification matrix stays in the shared
// memory of a thread-block cluster (CS CTAs, column slabs); a column never moves: the
// pivoting is tracked as a permutation (perm: position -> column, replicated in every
// CTA; pos: column -> position for the slab's own columns).  Per pivot step i:
//   1. every CTA reads the published (slab maximum m_q, first position f_q inside the tie
//      window of m_q) of all slabs and derives the pivot; exact as long as no slab maximum
//      lies inside the tie window below the global one (else one more barrier);
//   2. every CTA reads the pivot column through distributed shared memory and builds the
//      Householder reflector itself (identical arithmetic in every CTA);
//   3. every CTA applies the reflector to its trailing columns (G threads per column) and
//      downdates their norms (LAWN 176), then publishes its next (m, f) and arrives at the
//      cluster barrier.
// The owner writes the reflector into the pivot column one step later, once no CTA can
// still be reading that column.  At the end the slabs are written to the global workspace
// in LAPACK's column order (position p holds column perm[p]).
__device__ __forceinline__ void qc_barrier(cooperative_groups::cluster_group& cl, int cs) {
    if (cs > 1) cl.sync();
    else __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(QC_THREADS) qrcp_smem_kernel(Ctx<T> c, const DSpars* __restrict__ items,
                                                               const DAsn* __restrict__ pieces, T* ws, int* jpvt_ws,
                                                               int* ipvt_ws, T* taus, int* rank_out, int* colcount,
                                                               int* fallback, double tol, int smem_bytes,
                                                               unsigned long long* probe) {
    namespace cgx = cooperative_groups;
    cgx::cluster_group cl = cgx::this_cluster();
    const int CS = (int)cl.num_blocks();
    const int me = (int)cl.block_rank();
    const int item = blockIdx.x / CS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ T red[32];
    __shared__ int ired[32];
    __shared__ T pubm[2][16];
    __shared__ int pubf[2][16];
    __shared__ T s_alpha;
    if (c.status->not_spd) return;
    const DSpars it = items[item];
    const int rows = c.csize[it.cluster];
    int cols = 0;
    for (int p = 0; p < it.count; p++) cols += c.csize[pieces[it.first + p].nbr];
    const int mn = min(rows, cols);
    const int cpc = (cols + CS - 1) / CS;
    const int lda = rows | 1;
    const bool fits = qc_need(rows, cols, CS, (int)sizeof(T)) <= smem_bytes;
    if (threadIdx.x == 0 && me == 0) {
        fallback[item] = (mn > 0 && tol < 1.0 && !fits) ? 1 : 0;
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
    T* A = reinterpret_cast<T*>(smem_raw);
    T* vsh = A + (size_t)lda * cpc;
    T* vn1 = vsh + rows;
    T* vn2 = vn1 + cpc;
    int* perm = reinterpret_cast<int*>(vn2 + cpc);
    int* pos = perm + cols;
    const int c0 = me * cpc;
    const int c1 = min(cols, c0 + cpc);
    const int nloc = max(0, c1 - c0);
    const int tid = threadIdx.x, nth = blockDim.x;
    const int lane = tid & 31, w = tid >> 5, nw = nth >> 5;
    // gather the slab of Asn = [A_sn | A_ns^T]
    {
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
                        int i = idx % rows, jj = idx / rows;
                        A[i + (size_t)(lo - c0 + jj) * lda] = B[i + (size_t)(lo - col + jj) * bld];
                    }
                } else {
                    for (int idx = tid; idx < rows * width; idx += nth) {
                        int jj = idx % width, i = idx / width;
                        A[i + (size_t)(lo - c0 + jj) * lda] = B[(lo - col + jj) + (size_t)i * bld];
                    }
                }
            }
            col += n;
        }
    }
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
    // threads per column for the trailing update
    int G = 1;
    while (G < 8 && (nloc * G * 2 <= nth || rows >= 64 * G)) G *= 2;
    const int gid = tid / G, gl = tid % G, ngroups = nth / G;
    const T tie = T(1) - qrcp_tie<T>();
    const T tol3z = dsqrt(sizeof(T) == 8 ? T(2.220446049250313e-16) : T(1.1920929e-07));

    // publish (slab max over columns at positions >= from, first position inside its tie window)
    auto publish = [&](int par, int from) {
        __syncthreads();
        T m = 0;
        for (int j = tid; j < nloc; j += nth)
            if (pos[j] >= from) m = fmax(m, vn1[j]);
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) red[w] = m;
        __syncthreads();
        m = red[0];
        for (int k = 1; k < nw; k++) m = fmax(m, red[k]);
        int f = INT_MAX;
        for (int j = tid; j < nloc; j += nth)
            if (pos[j] >= from && vn1[j] >= m * tie) f = min(f, pos[j]);
        for (int o = 16; o > 0; o >>= 1) f = min(f, __shfl_xor_sync(0xffffffffu, f, o));
        if (lane == 0) ired[w] = f;
        __syncthreads();
        if (tid == 0) {
            for (int k = 1; k < nw; k++) f = min(f, ired[k]);
            f = min(f, ired[0]);
            for (int q = 0; q < CS; q++) {
                *cl.map_shared_rank(&pubm[par][me], q) = m;
                *cl.map_shared_rank(&pubf[par][me], q) = f;
            }
        }
    };

    // phase probe: cycles accumulated in registers, added to probe[] once at the end
    const bool probing = probe && item == 0 && me == 0 && tid == 0;
    long long tmark = probing ? clock64() : 0;
    unsigned long long pacc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    auto mark = [&](int k) {
        if (probing) {
            long long t = clock64();
            pacc[k] += (unsigned long long)(t - tmark);
            tmark = t;
        }
    };
    publish(0, 0);
    qc_barrier(cl, CS);
    mark(0);
    int rank = mn;
    T r00 = 0;
    int pend = -1;        // local column awaiting its reflector
    T pend_beta = 0;
    int pend_i = 0;
    for (int i = 0; i < mn; i++) {
        const int par = i & 1;
        T gmax = 0;
        for (int q = 0; q < CS; q++) gmax = fmax(gmax, pubm[par][q]);
        bool amb = false;
        for (int q = 0; q < CS; q++) amb |= (pubm[par][q] < gmax && pubm[par][q] >= gmax * tie);
        int pvt = INT_MAX;
        if (!amb) {
            for (int q = 0; q < CS; q++)
                if (pubm[par][q] == gmax) pvt = min(pvt, pubf[par][q]);
        } else {
            // a slab maximum inside the tie window below the global one: search every slab
            // with the global threshold
            int f = INT_MAX;
            for (int j = tid; j < nloc; j += nth)
                if (pos[j] >= i && vn1[j] >= gmax * tie) f = min(f, pos[j]);
            for (int o = 16; o > 0; o >>= 1) f = min(f, __shfl_xor_sync(0xffffffffu, f, o));
            if (lane == 0) ired[w] = f;
            __syncthreads();
            if (tid == 0) {
                for (int k = 0; k < nw; k++) f = min(f, ired[k]);
                for (int q = 0; q < CS; q++) *cl.map_shared_rank(&pubf[par][me], q) = f;
            }
            qc_barrier(cl, CS);
            for (int q = 0; q < CS; q++) pvt = min(pvt, pubf[par][q]);
        }
        if (pvt < i || pvt >= cols) pvt = i;  // all norms NaN: keep the current position
        mark(1);
        const int phys = perm[pvt];
        const int phys_i = perm[i];
        const int own = phys / cpc, lj = phys - own * cpc;
        // reflector of the previous step into its column (no CTA reads it any more)
        if (pend >= 0) {
            T* a = A + (size_t)pend * lda;
            for (int r = pend_i + 1 + tid; r < rows; r += nth) a[r] = vsh[r];
            if (tid == 0) a[pend_i] = pend_beta;
            pend = -1;
        }
        __syncthreads();
        mark(2);
        // pivot column -> vsh (rows >= i)
        const T* src = (own == me ? A : cl.map_shared_rank(A, own)) + (size_t)lj * lda;
        T part = 0;
        for (int r = i + tid; r < rows; r += nth) {
            const T v = src[r];
            if (r == i) {
                s_alpha = v;
                vsh[r] = T(1);
            } else {
                vsh[r] = v;
                part += v * v;
            }
        }
        part = warp_sum(part);
        if (lane == 0) red[w] = part;
        __syncthreads();
        T xnorm2 = 0;
        for (int k = 0; k < nw; k++) xnorm2 += red[k];
        const T alpha = s_alpha;
        const T xnorm = dsqrt(xnorm2);
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
        const T rii = fabs(beta);
        if (i == 0) r00 = rii;
        if (tol != 0.0 && i >= 1 && !(rii / r00 >= T(tol))) {
            rank = i;
            break;
        }
        if (tu != T(0))
            for (int r = i + 1 + tid; r < rows; r += nth) vsh[r] *= sc;
        if (me == 0 && tid == 0) taus[it.tau_off + i] = tu;
        __syncthreads();  // vsh final; every thread has read perm
        mark(3);
        if (tid == 0) {
            perm[i] = phys;
            perm[pvt] = phys_i;
        }
        // trailing update of this slab's columns and their norms; positions after the swap.
        // The loop runs the same number of times in every thread so that the group
        // shuffles always see all 32 lanes.  The first lane of each group also keeps the
        // largest new norm of its columns for the next pivot search.
        T mloc = 0;
        for (int base = 0; base < nloc; base += ngroups) {
            const int j = base + gid;
            const int ph = c0 + j;
            const bool active = j < nloc && ph != phys && pos[j] >= i;
            T* aj = A + (size_t)(active ? j : 0) * lda;
            T s = 0;
            if (active && tu != T(0)) {
                // four independent partial sums so the shared-memory loads overlap
                T s0 = 0, s1 = 0, s2 = 0, s3 = 0;
                int r = i + gl;
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
            if (active && tu != T(0)) {
                s *= tu;
                int r = i + gl;
                for (; r + 3 * G < rows; r += 4 * G) {
                    const T a0 = aj[r], a1 = aj[r + G], a2 = aj[r + 2 * G], a3 = aj[r + 3 * G];
                    aj[r] = a0 - s * vsh[r];
                    aj[r + G] = a1 - s * vsh[r + G];
                    aj[r + 2 * G] = a2 - s * vsh[r + 2 * G];
                    aj[r + 3 * G] = a3 - s * vsh[r + 3 * G];
                }
                for (; r < rows; r += G) aj[r] -= s * vsh[r];
            }
            __syncwarp();
            // norm downdating (LAWN 176), decided by the group's first lane
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
        mark(4);
        if (own == me) {
            pend = lj;
            pend_beta = beta;
            pend_i = i;
        }
        if (i + 1 < mn) {
            // publish (slab maximum, first position inside its tie window) for step i+1;
            // every thread rescans only the columns it updated itself
            for (int o = 16; o > 0; o >>= 1) mloc = fmax(mloc, __shfl_xor_sync(0xffffffffu, mloc, o));
            if (lane == 0) red[w] = mloc;
            __syncthreads();
            T m = red[0];
            for (int k = 1; k < nw; k++) m = fmax(m, red[k]);
            int f = INT_MAX;
            if (gl == 0)
                for (int j = gid; j < nloc; j += ngroups)
                    if (pos[j] > i && vn1[j] >= m * tie) f = min(f, pos[j]);
            for (int o = 16; o > 0; o >>= 1) f = min(f, __shfl_xor_sync(0xffffffffu, f, o));
            if (lane == 0) ired[w] = f;
            __syncthreads();
            if (tid == 0) {
                for (int k = 0; k < nw; k++) f = min(f, ired[k]);
                for (int q = 0; q < CS; q++) {
                    *cl.map_shared_rank(&pubm[par ^ 1][me], q) = m;
                    *cl.map_shared_rank(&pubf[par ^ 1][me], q) = f;
                }
            }
            mark(5);
            qc_barrier(cl, CS);
            mark(6);
        }
        if (probing) pacc[7] += 1;
    }
    if (probing)
        for (int k = 0; k < 8; k++) probe[k] += pacc[k];
    if (pend >= 0) {
        __syncthreads();
        T* a = A + (size_t)pend * lda;
        for (int r = pend_i + 1 + tid; r < rows; r += nth) a[r] = vsh[r];
        if (tid == 0) a[pend_i] = pend_beta;
    }
    // no CTA leaves while another may still read its shared memory
    qc_barrier(cl, CS);
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
QcKernel<T> qrcp_smem_kernel_ptr() {
    return qrcp_smem_kernel<T>;
}

template QcKernel<float> qrcp_smem_kernel_ptr<float>();
template QcKernel<double> qrcp_smem_kernel_ptr<double>();

}  // namespace spand

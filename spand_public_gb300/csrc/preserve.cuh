// Preservation (the reference's "phi" vectors, src/tree.cpp:1226-1409, 980-1002,
// 807-827, 1115-1128): the sparsification keeps the columns of a user matrix phi in the
// range of every compressed cluster, so that the preconditioner reproduces them exactly.
// Launchers of the device kernels; the kernels live in preserve.cu.
#pragma once

#include "kcommon.cuh"

namespace spand {

// Per-cluster restriction of phi: cluster c's block at phis + off[c], cap[c] x nphi,
// column-major with leading dimension cap[c].
template <typename T>
struct PhiCtx {
    T* phis;
    const long long* off;
    int nphi;
};

// phi_ = P^T phi split over the leaf clusters (tree.cpp:1477-1485): permuted row q goes to
// phis[dst[q] + j * ld[q]], from phinat[perm[q] + j * n] (natural ordering, FP64).
template <typename T>
void preserve_init(PhiCtx<T> P, const double* phinat, int n, const int* perm, const long long* dst, const int* ld,
                   cudaStream_t s);

// phi <- L^T phi (LLT, tree.cpp:807-809) or L^T P^T phi (LDLT, tree.cpp:824-827; perm_store
// != nullptr) of every scaled cluster, L in the lower triangle of its pivot block; tmp: a
// scratch laid out as phis.
template <typename T>
void preserve_scale(Ctx<T> c, PhiCtx<T> P, T* tmp, const int* clusters, const int* pivots, int count,
                    const int* perm_store, const long long* poff, cudaStream_t s);

// Parents' phi = their children's stacked at the merge offsets (tree.cpp:1115-1128).
template <typename T>
void preserve_merge(Ctx<T> c, PhiCtx<T> P, const int* parents, int np, const int* child_ptr, const int* child_idx,
                    const int* cpos, cudaStream_t s);

// Per sparsified cluster: [A_sn phi_n | A_ns^T phi_n] (pivot group included, signs for the
// LDLT sign pivot) and its QR.  adaptive = false (tol > 1, tree.cpp:1257-1287): the
// reflectors are the cluster's Q, rank = column count (rows when that is >= rows).
// adaptive = true (tree.cpp:1350-1370): Q1 = the explicit orthonormal basis, rank1 = its
// column count (rows when nothing is left to compress).  Both in vstore at the item's v_off.
template <typename T>
void preserve_basis(Ctx<T> c, PhiCtx<T> P, const DSpars* items, int n, const DAsn* pieces, const T* signs,
                    const long long* soff, T* vstore, T* tauws, int* rank1, int* rank, bool adaptive, cudaStream_t s);

// tree.cpp:1371-1405 after the QRCP of (I - Q1 Q1^T) Asn (rank2 in rank[]): Q2 from its
// reflectors, Q = the reflectors of the QR of [Q1 Q2] into vstore / tauws, rank = rank1 +
// rank2 (rows when that reaches rows).
template <typename T>
void preserve_combine(Ctx<T> c, const DSpars* items, int n, const T* ws, T* vstore, T* tauws, const int* rank1,
                      int* rank, cudaStream_t s);

// tree.cpp:993-1064 with pred == false: Q^T on phi and on every edge block of the cluster
// (in-edges from the left, out-edges from the right), the first rank rows / columns kept;
// the cluster's size becomes rank.  Q in the blocked WY form of the solve: reflectors in
// vstore, the T factors (sparsify_wy_kernel) in tstore.  ytiles: CTAs per item
// (preserve_apply_tiles).
template <typename T>
void preserve_apply(Ctx<T> c, PhiCtx<T> P, const DSpars* items, int n, int ytiles, const DAsn* pieces,
                    const T* vstore, const T* tstore, const int* rank, cudaStream_t s);

// CTAs per item of preserve_apply: 32-vector tiles of the pieces' capacities and of phi
int preserve_apply_tiles(const int* caps, int count, int nphi);

// LoRaSp split (tree.cpp:1018-1064 with keep_sibling): Q^T (blocked WY form, T factors in
// tstore) on every original edge of each item, rows rank .. rows-1 copied into the sibling's
// block; sibling sizes set.  sibs / ranges: per item its sibling and its slice of splits
// (block, neighbour, transposed, sibling block).  ytiles: lorasp_split_tiles.
template <typename T>
void lorasp_split(Ctx<T> c, const DSpars* items, int n, int ytiles, const int* sibs, const int2* ranges,
                  const int4* splits, const T* vstore, const T* tstore, const int* rank, cudaStream_t s);
int lorasp_split_tiles(const int* caps, int count);

}  // namespace spand

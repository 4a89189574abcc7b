// Host side of the GB300 spaND path: ordering, assembly and the symbolic plan.
//
// The reference (leopoldcambier/spaND_public) runs partition / assemble / factorize /
// solve in one host thread on Eigen blocks.  Here the host keeps the nested-dissection
// ordering and cluster tree (bit-exact with src/partition.cpp and src/tree.cpp:306-419)
// and the assembly (src/tree.cpp:505-575), then replays the factorization's *structure*
// once.  The structure (which clusters are eliminated, scaled, sparsified and merged,
// which fill-in blocks appear, the order of every Schur update) does not depend on the
// QRCP ranks; only block sizes do.  The replay therefore yields a static plan of integer
// work lists; the device runs the numeric factorization from that plan with the cluster
// sizes kept in device memory, so the whole factorization is a fixed launch sequence.
#pragma once

#include <array>
#include <cstdint>
#include <list>
#include <string>
#include <vector>

namespace spand {

struct SepID {
    int lvl = -1, sep = 0;
    SepID() {}
    SepID(int l, int s) : lvl(l), sep(s) {}
    bool operator==(const SepID& o) const { return lvl == o.lvl && sep == o.sep; }
    bool operator!=(const SepID& o) const { return !(*this == o); }
    bool operator<(const SepID& o) const { return lvl < o.lvl || (lvl == o.lvl && sep < o.sep); }
};

struct ClusterID {
    SepID self, l, r;
    ClusterID() {}
    ClusterID(SepID s, SepID a, SepID b) : self(s), l(a), r(b) {}
    bool operator==(const ClusterID& o) const { return self == o.self && l == o.l && r == o.r; }
    bool operator!=(const ClusterID& o) const { return !(*this == o); }
    bool operator<(const ClusterID& o) const {
        if (!(self == o.self)) return self < o.self;
        if (!(l == o.l)) return l < o.l;
        return r < o.r;
    }
};

// Compressed sparse column matrix, sorted row indices, no duplicates.
struct Csc {
    int n = 0;
    std::vector<int> colptr, rowval;
    std::vector<double> val;
};

// Nested dissection (src/partition.cpp:384-478, geometric branch :139-210).
// X is dim x n, column-major.  Returns one ClusterID per dof (natural ordering).
std::vector<ClusterID> partition_modified_nd(const Csc& A, int nlevels, const double* X, int dim);

// Algebraic nested dissection through a METIS vertex separator (src/partition.cpp:51-97).
// Returns false when no METIS library can be loaded at run time.
bool partition_modified_nd_metis(const Csc& A, int nlevels, std::vector<ClusterID>& out, std::string& err);

// Block kinds of the plan.
enum BlockFlag : int { BLK_STORED = 0, BLK_IDENTITY = 1 };

// Device work items.  All sizes are read on the device from the per-cluster size
// array; the host fixes only identities, orders and storage capacities.
struct PlanBlock {
    int64_t off = 0;   // element offset in the block arena
    int ld = 0;        // leading dimension = capacity of the row cluster
    int rowc = -1;     // row cluster (edge n2)
    int colc = -1;     // column cluster (edge n1)
    int flag = BLK_STORED;
};

// One Schur update C(n1 x n2) -= X Y with X = op1(B1) (n1 x s), Y = op2(B2) (s x n2);
// the reference's gemm_edges (src/tree.cpp:748-793).
struct SchurUpdate {
    int b1, t1, b2, t2, s;  // blocks, transpose flags, eliminated cluster
};

struct SchurTarget {
    int target;     // target block
    int syrk;       // n1 == n2 on the symmetric path: lower triangle only (0 on the LU path)
    int first, count;  // slice of Plan::schur_updates, in reference order
};

// Triangular solve of a block by the factor of a cluster's pivot:
// side 0: B <- L^{-1} B (block rows belong to the cluster: in-edge); LU path: L^{-1} P^T B
// side 1: B <- B L^{-T} (block columns belong to the cluster: out-edge); LU path: B U^{-1}
struct TrsmItem {
    int block, cluster, side;
};

// One column group of a sparsification matrix Asn = [A_sn (in-edges) | A_ns^T (out-edges)]
// (src/tree.cpp:1189-1224).
struct AsnPiece {
    int block, nbr, transposed;
};

struct SparsifyItem {
    int cluster;
    int first, count;   // slice of Plan::asn_pieces
    int64_t ws_off;     // Asn workspace offset (elements) within the wave scratch
    int cap_cols;       // capacity of Asn columns
    int64_t v_off;      // persistent reflector storage (cap x cap) for the Orthogonal op
    int64_t tau_off;    // persistent tau storage (cap)
    // LDLT path (src/tree.cpp:1069-1097): the cluster's pivot block (sign(D) after its
    // scaling, transformed to Q^T D Q and split), the sibling cluster made of the dropped
    // rows, its pivot block and the block of the edge original -> sibling (-1 elsewhere)
    int piv = -1, sib = -1, sib_piv = -1, aso = -1;
    // LoRaSp (src/tree.cpp:1018-1064, keep_sibling): the original edges, slice of
    // Plan::lr_splits; the sibling's GemmSymmIn ops, slice of Plan::lr_sibops
    int ofirst = 0, ocount = 0, sfirst = 0, scount = 0;
};

// LoRaSp: an original edge of a sparsified cluster, Q^T-transformed, whose last rows go to
// the sibling's edge block sblock (sibling x neighbour)
struct LoraSplit {
    int block, nbr, transposed, sblock;
};

// LoRaSp: GemmSymmIn(sibling, nbr) with the block sibling x nbr; cur: the neighbour was
// sparsified earlier in the level (its size is then its rank)
struct LoraSibOp {
    int nbr, block, cur;
};

// Copy of a child block into a parent block during a merge (src/tree.cpp:1133-1184).
struct MergeCopy {
    int src;    // source block (BLK_IDENTITY: write an identity of the child size)
    int dst;    // parent block
    int nold;   // child cluster giving the row offset
    int sold;   // child cluster giving the column offset
};

// Solve-time operations, grouped per level and phase (src/operations.cpp:31-208).
struct GemmOpItem {
    // kind 1: GemmSymmOut (A: nbr x self), 2: GemmSymmIn (A: self x nbr); LU path:
    // 6: GemmOut (A: nbr x self, forward only), 7: GemmIn (A: self x nbr, backward only)
    int self, nbr, block, kind;
};

struct LevelPlan {
    // elimination (src/tree.cpp:1494-1506)
    std::vector<int> elim_clusters;
    std::vector<int> elim_pivots;
    std::vector<int> elim_inv;  // LU path: block of the pivot's inverse factors (else -1)
    std::vector<TrsmItem> elim_trsm;
    int schur_first = 0, schur_count = 0;  // slice of Plan::schur_targets
    int64_t fill_off = 0, fill_len = 0;    // zero-initialised fill-in region
    // scaling (src/tree.cpp:1510-1519)
    bool scaled = false;
    std::vector<int> scale_clusters;
    std::vector<int> scale_pivots;
    std::vector<int> scale_inv;
    std::vector<int> scale_newpiv;  // LDLT: block receiving diag(sign D) as the new pivot
    std::vector<TrsmItem> scale_trsm;
    // sparsification (src/tree.cpp:1521-1532): waves of mutually non-adjacent clusters
    std::vector<std::vector<SparsifyItem>> waves;
    int64_t ws_len = 0;  // workspace elements needed by the largest wave
    int ignored = 0;
    // merge (src/tree.cpp:1536-1543)
    bool merged = false;
    std::vector<int> merge_parents;
    std::vector<MergeCopy> merge_copies;
    int64_t merge_off = 0, merge_len = 0;
    // solve operations recorded at this level
    std::vector<int> op_elim_llt;         // eliminated clusters (ScalingLLT / ScalingPLUQ of the pivot block)
    std::vector<int> op_elim_llt_block;
    std::vector<GemmOpItem> op_gemm;      // in reference order
    std::vector<int> op_scale_llt;        // scaled clusters
    std::vector<int> op_scale_llt_block;
    std::vector<int> op_ortho;            // sparsified clusters (Orthogonal if rank < rows)
    std::vector<int> op_merge;            // parents
    // LoRaSp: each wave of a level is a level of the plan; real: the reference's level,
    // snap: the clusters whose size is recorded at its start (the wave's own)
    int real = -1;
    std::vector<int> snap;
};

struct Plan {
    int nlevels = 0;
    // LU path (SymmKind::GEN, ScalingKind::PLU): every stored block in both directions,
    // partial-pivot LU of the pivots, Schur updates over (out-edge, in-edge) pairs
    bool lu = false;
    // LDLT path (SymmKind::SYM, ScalingKind::LDLT): the symmetric structure with pivoted
    // LDL^T pivots, sign-weighted Schur updates, sign pivots after scaling and an explicit
    // sibling per sparsified cluster (clusters nclusters_h .. nclusters-1)
    bool ldlt = false;
    // LoRaSp (src/tree.cpp:1553-1608): no interior elimination; every cluster is scaled and
    // sparsified over its fill-in edges only, its sibling keeps the original edges and is
    // eliminated right away (explicit siblings, as on the LDLT path)
    bool lorasp = false;
    std::vector<LoraSplit> lr_splits;
    std::vector<LoraSibOp> lr_sibops;
    // per reference level: the clusters in processing order, with their plan level and item
    std::vector<std::vector<std::array<int, 3>>> lr_order;  // (cluster, plan level, item index in its wave)
    int nclusters_h = 0;  // clusters of the hierarchy; the rest are LDLT siblings
    int nclusters = 0;        // clusters of the hierarchy (siblings are implicit)
    std::vector<int> c_start, c_cap, c_level, c_order, c_hlevel, c_parent, c_sparsify;
    std::vector<std::vector<int>> c_children;
    std::vector<int64_t> c_xoff;  // solve-vector slot (capacity c_cap)
    int64_t x_len = 0;
    std::vector<PlanBlock> blocks;
    std::vector<int> initial_blocks;  // blocks filled by assembly
    int64_t arena_len = 0;            // elements
    int64_t assembled_len = 0;        // elements [0, assembled_len) hold the assembled level-0 blocks
    std::vector<SchurUpdate> schur_updates;
    std::vector<SchurTarget> schur_targets;
    std::vector<AsnPiece> asn_pieces;
    int64_t v_len = 0, tau_len = 0;
    int64_t ws_len = 0;  // max over waves
    std::vector<LevelPlan> levels;
    // structural statistics
    int64_t n_fill_blocks = 0, n_merge_blocks = 0;
};

// The symbolic replay of Tree::factorize (src/tree.cpp:1447-1551) for the LLT path, or
// for the PLU path (lu: general matrices, src/tree.cpp:614-742, 929-956).
// leaves: per leaf cluster (start, size, level, order, sparsify); the hierarchy through
// parent/children; assembled leaf blocks come from assemble().
struct Hierarchy {
    int nlevels = 0;
    std::vector<int> start, size, level, sparsify, parent, hlevel;
    std::vector<std::vector<int>> children;
    std::vector<std::vector<int>> bottoms;  // per hierarchy level: cluster ids in list order
};

Hierarchy build_hierarchy(const std::vector<ClusterID>& part, int nlevels, std::vector<int>& perm);

// LoRaSp ordering: geometric recursive bisection (src/partition.cpp:99-137, 245-285), the part
// of every dof (natural ordering); X is dim x n, column-major
std::vector<int> partition_rb(int n, int nlevels, const double* X, int dim);
// LoRaSp hierarchy (src/tree.cpp:421-503): every cluster at the top level, pairs of
// consecutive clusters merge; perm: the assembly permutation (sort by part)
Hierarchy build_hierarchy_lorasp(const std::vector<int>& parts, int nlevels, std::vector<int>& perm);

// Assembly: per leaf cluster, the sorted neighbour list (pivot first) and the dense
// blocks (src/tree.cpp:505-575).  values is laid out with the plan's block offsets.
struct Assembly {
    std::vector<std::vector<int>> nbrs;  // per leaf: neighbour clusters, sorted by order, self first
};
Assembly assembly_structure(const Hierarchy& H, const Csc& App, bool symmetric);

Plan build_plan(const Hierarchy& H, const Assembly& asmb, int skip, bool use_want_sparsify, bool lu = false,
                bool ldlt = false);
// The symbolic replay of Tree::factorize_lorasp (src/tree.cpp:1553-1608), SPD / LLT
Plan build_plan_lorasp(const Hierarchy& H, const Assembly& asmb);

// For every entry k of A (natural ordering, CSC order): the element offset of A(r, c) in
// the assembled level-0 blocks, or -1 when the entry is not stored (upper triangle of the
// symmetric path).  Reproduces block2dense (util.cpp:454-486) on A[p,p] as a gather map,
// so that re-assembly with new values is one scatter on the device.
std::vector<int64_t> assembly_map(const Plan& P, const Hierarchy& H, const Assembly& asmb, const Csc& A,
                                  const std::vector<int>& perm);

Csc symm_perm(const Csc& A, const std::vector<int>& perm);

}  // namespace spand

// Host side of the GB300 spaND path: ordering, assembly structure and the symbolic plan.
// See host.h for the design.  Citations are path:line into leopoldcambier/spaND_public.
#include "host.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <numeric>
#include <set>
#include <stdexcept>

#include <dlfcn.h>

namespace spand {

// ------------------------------------------------------------------------------------
// Ordering
// ------------------------------------------------------------------------------------

static SepID sep_merge(const SepID& s) { return SepID(s.lvl + 1, s.sep / 2); }

// partition.cpp:12-16
static ClusterID merge_if(const ClusterID& c, int lvl) {
    return ClusterID(c.self, c.l.lvl < lvl ? sep_merge(c.l) : c.l, c.r.lvl < lvl ? sep_merge(c.r) : c.r);
}

namespace {

// Adjacency without self loops (partition.cpp:21-39).
struct Graph {
    std::vector<int> ptr, adj;
};

Graph graph_of(const Csc& A) {
    Graph G;
    G.ptr.assign(A.n + 1, 0);
    G.adj.reserve(A.rowval.size());
    for (int j = 0; j < A.n; j++) {
        for (int k = A.colptr[j]; k < A.colptr[j + 1]; k++)
            if (A.rowval[k] != j) G.adj.push_back(A.rowval[k]);
        G.ptr[j + 1] = (int)G.adj.size();
    }
    return G;
}

// One geometric bisection with a one-sided vertex separator (partition.cpp:139-210):
// split the widest coordinate at the median value (strictly below goes left), then
// every right-side dof that touches the left side joins the separator.
// side[i] in {0: left, 1: right, 2: separator} for dofs[i].
void geo_bisect(const Graph& G, const std::vector<int>& dofs, const double* X, int dim, std::vector<int>& side,
                std::vector<int>& local) {
    const int N = (int)dofs.size();
    side.assign(N, 0);
    if (N == 0) return;
    int axis = -1;
    double widest = -1.0;
    for (int d = 0; d < dim; d++) {
        double lo = std::numeric_limits<double>::max(), hi = std::numeric_limits<double>::lowest();
        for (int v : dofs) {
            double x = X[d + (size_t)dim * v];
            lo = std::min(lo, x);
            hi = std::max(hi, x);
        }
        if (hi - lo > widest) { widest = hi - lo; axis = d; }
    }
    std::vector<double> coord(N);
    for (int i = 0; i < N; i++) coord[i] = X[axis + (size_t)dim * dofs[i]];
    std::vector<double> tmp(coord);
    std::nth_element(tmp.begin(), tmp.begin() + N / 2, tmp.end());
    const double cut = tmp[N / 2];
    // local index of every dof of this subdomain, -1 for its outside neighbours
    for (int i = 0; i < N; i++) {
        int v = dofs[i];
        local[v] = -1;
        for (int k = G.ptr[v]; k < G.ptr[v + 1]; k++) local[G.adj[k]] = -1;
    }
    for (int i = 0; i < N; i++) {
        local[dofs[i]] = i;
        side[i] = coord[i] < cut ? 0 : 1;
    }
    for (int i = 0; i < N; i++) {
        if (side[i] == 0) continue;
        int v = dofs[i];
        for (int k = G.ptr[v]; k < G.ptr[v + 1]; k++) {
            int li = local[G.adj[k]];
            if (li >= 0 && side[li] == 0) { side[i] = 2; break; }
        }
    }
}

// Apply one bisection result to the (self, left, right) labels and return the two child
// subdomains (partition.cpp:421-470).  Separator dofs of ancestors stay in both children.
void relabel(std::vector<ClusterID>& part, const std::vector<int>& dofs, const std::vector<int>& side, int level,
             int sep, std::vector<int>& left, std::vector<int>& right) {
    const SepID me(level, sep), lo(level - 1, 2 * sep), hi(level - 1, 2 * sep + 1);
    for (size_t i = 0; i < dofs.size(); i++) {
        ClusterID& c = part[dofs[i]];
        const int s = side[i];
        if (s == 2) {
            if (c.self == me) { c.l = lo; c.r = hi; }
            continue;
        }
        const SepID to = s == 0 ? lo : hi;
        if (c.self == me) c.self = to;
        if (c.l == me) c.l = to;
        if (c.r == me) c.r = to;
    }
    left.clear();
    right.clear();
    for (int v : dofs) {
        const ClusterID& c = part[v];
        if (c.self == lo || c.l == lo || c.r == lo) left.push_back(v);
        if (c.self == hi || c.l == hi || c.r == hi) right.push_back(v);
    }
}

}  // namespace

std::vector<ClusterID> partition_modified_nd(const Csc& A, int nlevels, const double* X, int dim) {
    const int N = A.n;
    Graph G = graph_of(A);
    const SepID top(nlevels - 1, 0);
    std::vector<ClusterID> part(N, ClusterID(top, top, top));
    std::vector<std::vector<int>> doms(1);
    doms[0].resize(N);
    std::iota(doms[0].begin(), doms[0].end(), 0);
    std::vector<int> local(N + 1, -1), side;
    for (int depth = 0; depth + 1 < nlevels; depth++) {
        const int level = nlevels - 1 - depth;
        std::vector<std::vector<int>> next(doms.size() * 2);
        for (size_t sep = 0; sep < doms.size(); sep++) {
            std::vector<int> dofs = doms[sep];
            std::sort(dofs.begin(), dofs.end());
            geo_bisect(G, dofs, X, dim, side, local);
            relabel(part, dofs, side, level, (int)sep, next[2 * sep], next[2 * sep + 1]);
        }
        doms.swap(next);
    }
    return part;
}

// --- METIS (algebraic ordering), loaded at run time --------------------------------
// The reference calls METIS_ComputeVertexSeparator on the subdomain graph
// (partition.cpp:51-97).  METIS is optional here: the GB300 image ships a static
// libmetis only, so algebraic ordering is available when a shared libmetis.so is found.
bool partition_modified_nd_metis(const Csc& A, int nlevels, std::vector<ClusterID>& out, std::string& err) {
    void* h = dlopen("libmetis.so", RTLD_NOW | RTLD_LOCAL);
    if (!h) {
        err = "algebraic ordering needs libmetis.so, which is not available; pass grid coordinates (set_Xcoo)";
        return false;
    }
    dlclose(h);
    err = "algebraic ordering through METIS is not available in this library; pass grid coordinates (set_Xcoo)";
    (void)A;
    (void)nlevels;
    (void)out;
    return false;
}

// ------------------------------------------------------------------------------------
// Cluster hierarchy (tree.cpp:336-415)
// ------------------------------------------------------------------------------------
Hierarchy build_hierarchy(const std::vector<ClusterID>& part, int nlevels, std::vector<int>& perm) {
    const int N = (int)part.size();
    Hierarchy H;
    H.nlevels = nlevels;
    H.bottoms.resize(nlevels);
    // ordering: stable sorts by the ID, then by the ID merged up to every level
    perm.resize(N);
    std::iota(perm.begin(), perm.end(), 0);
    std::vector<ClusterID> key(part);
    auto by_key = [&key](int a, int b) { return key[a] < key[b]; };
    std::stable_sort(perm.begin(), perm.end(), by_key);
    for (int lvl = 1; lvl < nlevels; lvl++) {
        for (auto& k : key) k = merge_if(k, lvl);
        std::stable_sort(perm.begin(), perm.end(), by_key);
    }
    std::vector<ClusterID> cid;  // per cluster
    auto add = [&](int start, int size, int level, bool sp, int hl) {
        H.start.push_back(start);
        H.size.push_back(size);
        H.level.push_back(level);
        H.sparsify.push_back(sp ? 1 : 0);
        H.parent.push_back(-1);
        H.hlevel.push_back(hl);
        H.children.emplace_back();
        return (int)H.start.size() - 1;
    };
    // leaves: runs of equal (unmerged) ID in the permuted order
    for (int k = 0; k < N;) {
        const ClusterID id = part[perm[k]];
        int e = k + 1;
        while (e < N && part[perm[e]] == id) e++;
        int c = add(k, e - k, id.self.lvl, id.l.lvl == 0 && id.r.lvl == 0, 0);
        cid.push_back(id);
        H.bottoms[0].push_back(c);
        k = e;
    }
    for (int lvl = 1; lvl < nlevels; lvl++) {
        const std::vector<int>& prev = H.bottoms[lvl - 1];
        size_t b = 0;
        while (b < prev.size() && H.level[prev[b]] < lvl) b++;
        std::vector<ClusterID> pid(prev.size());
        for (size_t i = b; i < prev.size(); i++) pid[i] = merge_if(cid[prev[i]], lvl);
        for (size_t i = b; i < prev.size();) {
            size_t e = i + 1;
            int size = H.size[prev[i]];
            while (e < prev.size() && pid[e] == pid[i]) size += H.size[prev[e++]];
            const ClusterID& p = pid[i];
            int c = add(H.start[prev[i]], size, p.self.lvl, p.l.lvl == lvl && p.r.lvl == lvl, lvl);
            cid.push_back(p);
            for (size_t j = i; j < e; j++) {
                H.parent[prev[j]] = c;
                H.children[c].push_back(prev[j]);
            }
            H.bottoms[lvl].push_back(c);
            i = e;
        }
    }
    return H;
}

// ------------------------------------------------------------------------------------
// LoRaSp ordering and hierarchy
// ------------------------------------------------------------------------------------
// partition.cpp:99-137: the widest coordinate of the part, cut at the value of its middle
// dof in that coordinate (dofs at or below it go to part start, the others to start + 1)
static void rb_bisect(const std::vector<int>& dofs, std::vector<int>& parts, const double* X, int dim, int start) {
    const int N = (int)dofs.size();
    if (N == 0) return;
    int axis = -1;
    double widest = -1.0;
    for (int d = 0; d < dim; d++) {
        double hi = std::numeric_limits<double>::lowest(), lo = std::numeric_limits<double>::max();
        for (int v : dofs) {
            hi = std::max(hi, X[d + (size_t)dim * v]);
            lo = std::min(lo, X[d + (size_t)dim * v]);
        }
        if (hi - lo > widest) {
            widest = hi - lo;
            axis = d;
        }
    }
    std::vector<double> coord(N);
    for (int i = 0; i < N; i++) coord[i] = X[axis + (size_t)dim * dofs[i]];
    std::nth_element(coord.begin(), coord.begin() + N / 2, coord.end());
    const double cut = coord[N / 2];  // the value of the middle dof once sorted
    for (int v : dofs) parts[v] = X[axis + (size_t)dim * v] <= cut ? start : start + 1;
}

// partition.cpp:245-285, geometric branch
std::vector<int> partition_rb(int n, int nlevels, const double* X, int dim) {
    std::vector<int> parts(n, 0);
    for (int depth = 0; depth + 1 < nlevels; depth++) {
        const int np = 1 << depth;
        std::vector<std::vector<int>> dofs(np);
        for (int i = 0; i < n; i++) dofs[parts[i]].push_back(i);
        for (int k = 0; k < np; k++) rb_bisect(dofs[k], parts, X, dim, 2 * k);
    }
    return parts;
}

// tree.cpp:421-503.  The dofs are sorted by part with std::sort (not stable), as the
// reference does: the order inside a part is then that of the standard library's sort.
Hierarchy build_hierarchy_lorasp(const std::vector<int>& parts, int nlevels, std::vector<int>& perm) {
    const int N = (int)parts.size();
    Hierarchy H;
    H.nlevels = nlevels;
    H.bottoms.resize(nlevels);
    perm.resize(N);
    std::iota(perm.begin(), perm.end(), 0);
    std::sort(perm.begin(), perm.end(), [&parts](int i, int j) { return parts[i] < parts[j]; });
    const int top = nlevels - 1;
    std::vector<int> id;  // per cluster: its order (leaves), then the parent id (order / 2 upwards)
    auto add = [&](int start, int size, int hl) {
        H.start.push_back(start);
        H.size.push_back(size);
        H.level.push_back(top);
        H.sparsify.push_back(1);
        H.parent.push_back(-1);
        H.hlevel.push_back(hl);
        H.children.emplace_back();
        return (int)H.start.size() - 1;
    };
    for (int k = 0; k < N;) {
        int e = k + 1;
        while (e < N && parts[perm[e]] == parts[perm[k]]) e++;
        const int c = add(k, e - k, 0);
        id.push_back(c);
        H.bottoms[0].push_back(c);
        k = e;
    }
    for (int lvl = 1; lvl < nlevels; lvl++) {
        const std::vector<int>& prev = H.bottoms[lvl - 1];
        for (size_t i = 0; i < prev.size();) {
            const int pid = id[prev[i]] / 2;
            size_t e = i + 1;
            int size = H.size[prev[i]];
            while (e < prev.size() && id[prev[e]] / 2 == pid) size += H.size[prev[e++]];
            const int c = add(H.start[prev[i]], size, lvl);
            id.push_back(pid);
            for (size_t j = i; j < e; j++) {
                H.parent[prev[j]] = c;
                H.children[c].push_back(prev[j]);
            }
            H.bottoms[lvl].push_back(c);
            i = e;
        }
    }
    return H;
}

// A[p,p] (util.cpp:519-546)
Csc symm_perm(const Csc& A, const std::vector<int>& perm) {
    const int n = A.n;
    std::vector<int> pinv(n);
    for (int i = 0; i < n; i++) pinv[perm[i]] = i;
    Csc B;
    B.n = n;
    B.colptr.assign(n + 1, 0);
    for (int jn = 0; jn < n; jn++) {
        int j = perm[jn];
        B.colptr[jn + 1] = B.colptr[jn] + (A.colptr[j + 1] - A.colptr[j]);
    }
    B.rowval.resize(A.rowval.size());
    B.val.resize(A.val.size());
    std::vector<std::pair<int, double>> col;
    for (int jn = 0; jn < n; jn++) {
        int j = perm[jn];
        col.clear();
        for (int k = A.colptr[j]; k < A.colptr[j + 1]; k++) col.emplace_back(pinv[A.rowval[k]], A.val.empty() ? 0.0 : A.val[k]);
        std::sort(col.begin(), col.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
        int o = B.colptr[jn];
        for (size_t t = 0; t < col.size(); t++) {
            B.rowval[o + t] = col[t].first;
            B.val[o + t] = col[t].second;
        }
    }
    return B;
}

// Neighbour sets of the leaf clusters (tree.cpp:535-548): rows of the cluster's columns
// (lower triangle only on the symmetric path), plus the cluster itself.
Assembly assembly_structure(const Hierarchy& H, const Csc& App, bool symmetric) {
    Assembly out;
    const int N = App.n;
    std::vector<int> owner(N);
    for (int c : H.bottoms[0])
        for (int k = H.start[c]; k < H.start[c] + H.size[c]; k++) owner[k] = c;
    out.nbrs.resize(H.bottoms[0].size());
    for (size_t li = 0; li < H.bottoms[0].size(); li++) {
        int c = H.bottoms[0][li];
        std::set<int> s;
        s.insert(c);
        for (int j = H.start[c]; j < H.start[c] + H.size[c]; j++)
            for (int k = App.colptr[j]; k < App.colptr[j + 1]; k++) {
                int row = App.rowval[k];
                if (symmetric && row < j) continue;
                s.insert(owner[row]);
            }
        std::vector<int>& v = out.nbrs[li];
        v.push_back(c);
        for (int n : s)
            if (n != c) v.push_back(n);
    }
    return out;
}

// ------------------------------------------------------------------------------------
// Symbolic replay of Tree::factorize (LLT path)
// ------------------------------------------------------------------------------------
namespace {

struct SymEdge {
    int n1, n2, block;
};

struct SymTree {
    const Hierarchy& H;
    Plan& P;
    std::vector<SymEdge> edges;
    std::vector<char> orig;  // per edge: an original (assembled) coupling, or merged from one
    std::vector<std::list<int>> out, in;  // per cluster: edge ids (out: pivot first)
    std::vector<char> eliminated;

    SymTree(const Hierarchy& h, Plan& p) : H(h), P(p), out(h.start.size()), in(h.start.size()), eliminated(h.start.size(), 0) {}

    int new_block(int rowc, int colc, int flag, int64_t& cursor) {
        return new_block(rowc, colc, flag, cursor, P.c_cap[rowc], P.c_cap[colc]);
    }
    // with explicit row / column capacities (the sizes the block can reach from now on)
    int new_block(int rowc, int colc, int flag, int64_t& cursor, int rcap, int ccap) {
        PlanBlock b;
        b.rowc = rowc;
        b.colc = colc;
        b.flag = flag;
        b.ld = std::max(rcap, 1);
        if (flag == BLK_STORED) {
            b.off = cursor;
            cursor += (int64_t)b.ld * std::max(ccap, 0);
            cursor = (cursor + 31) & ~int64_t(31);  // 256-byte aligned blocks in FP64
        }
        P.blocks.push_back(b);
        return (int)P.blocks.size() - 1;
    }
    // cluster.cpp:113-123
    int add_edge(int n1, int n2, int block, bool original = true) {
        edges.push_back({n1, n2, block});
        orig.push_back(original ? 1 : 0);
        int e = (int)edges.size() - 1;
        if (n1 == n2) {
            out[n1].push_front(e);
        } else {
            in[n2].push_back(e);
            out[n1].push_back(e);
        }
        return e;
    }
    // cluster.cpp:161-176
    void sort_edges(int c) {
        out[c].sort([this](int a, int b) {
            const SymEdge& x = edges[a];
            const SymEdge& y = edges[b];
            if (x.n1 == x.n2) return true;
            if (y.n1 == y.n2) return false;
            return x.n2 < y.n2;
        });
        in[c].sort([this](int a, int b) { return edges[a].n1 < edges[b].n1; });
    }
    std::vector<int> out_nbr(int c) {
        std::vector<int> r;
        auto it = out[c].begin();
        if (it != out[c].end()) ++it;
        for (; it != out[c].end(); ++it) r.push_back(*it);
        return r;
    }
    std::vector<int> in_nbr(int c) { return std::vector<int>(in[c].begin(), in[c].end()); }
    int pivot(int c) { return out[c].front(); }
    // cluster.cpp:32-45
    void set_eliminated(int c) {
        for (int e : out[c]) {
            int n = edges[e].n2;
            if (n != c) in[n].remove_if([this, c](int e2) { return edges[e2].n1 == c; });
        }
        for (int e : in[c]) {
            int n = edges[e].n1;
            out[n].remove_if([this, c](int e2) { return edges[e2].n2 == c; });
        }
        out[c].clear();
        in[c].clear();
        eliminated[c] = 1;
    }
};

}  // namespace

Plan build_plan(const Hierarchy& H, const Assembly& asmb, int skip, bool use_want_sparsify, bool lu, bool ldlt) {
    Plan P;
    P.lu = lu;
    P.ldlt = ldlt;
    const int nl = H.nlevels;
    const int nc = (int)H.start.size();
    P.nlevels = nl;
    P.nclusters = nc;
    P.c_start = H.start;
    P.c_cap = H.size;
    P.c_level = H.level;
    P.c_hlevel = H.hlevel;
    P.c_parent = H.parent;
    P.c_sparsify = H.sparsify;
    P.c_children = H.children;
    P.c_order.resize(nc);
    std::iota(P.c_order.begin(), P.c_order.end(), 0);
    P.c_xoff.resize(nc);
    for (int c = 0; c < nc; c++) {
        P.c_xoff[c] = P.x_len;
        P.x_len += H.size[c];
    }
    SymTree T(H, P);
    int64_t cursor = 0;
    // Assembled leaf blocks (tree.cpp:549-559): nbr x self, pivot first then by order.
    for (size_t li = 0; li < H.bottoms[0].size(); li++) {
        int self = H.bottoms[0][li];
        for (int nbr : asmb.nbrs[li]) {
            int b = T.new_block(nbr, self, BLK_STORED, cursor);
            P.initial_blocks.push_back(b);
            T.add_edge(self, nbr, b);
        }
        T.sort_edges(self);
    }
    P.assembled_len = cursor;
    P.levels.resize(nl);
    std::map<int, std::vector<SchurUpdate>> pending;  // target block -> updates
    std::vector<int> target_order;
    std::vector<int> target_syrk;

    for (int ilvl = 0; ilvl < nl; ilvl++) {
        LevelPlan& L = P.levels[ilvl];
        const std::vector<int>& bottom = H.bottoms[ilvl];
        // ---- eliminate interiors (tree.cpp:895-967, LLT) ----
        L.fill_off = cursor;
        pending.clear();
        target_order.clear();
        target_syrk.clear();
        auto gemm_edges = [&](int e1, int e2, bool t1, bool t2) {  // tree.cpp:748-793
            const SymEdge E1 = T.edges[e1], E2 = T.edges[e2];
            int s = t1 ? E1.n2 : E1.n1;
            int n1 = t1 ? E1.n1 : E1.n2;
            int n2 = t2 ? E2.n2 : E2.n1;
            int found = -1;
            for (int e : T.out[n2])
                if (T.edges[e].n2 == n1) { found = e; break; }
            if (found < 0) {
                int b = T.new_block(n1, n2, BLK_STORED, cursor);
                found = T.add_edge(n2, n1, b);
                P.n_fill_blocks++;
            }
            int tb = T.edges[found].block;
            auto it = pending.find(tb);
            if (it == pending.end()) {
                target_order.push_back(tb);
                target_syrk.push_back(n1 == n2 && !lu ? 1 : 0);
                it = pending.emplace(tb, std::vector<SchurUpdate>()).first;
            }
            it->second.push_back({E1.block, t1 ? 1 : 0, E2.block, t2 ? 1 : 0, s});
        };
        for (int s : bottom) {
            if (H.level[s] != ilvl) continue;
            int piv = T.edges[T.pivot(s)].block;
            L.elim_clusters.push_back(s);
            L.elim_pivots.push_back(piv);
            L.elim_inv.push_back(lu ? T.new_block(s, s, BLK_STORED, cursor) : -1);
            auto ins = T.in_nbr(s);
            auto outs = T.out_nbr(s);
            for (int e : ins) L.elim_trsm.push_back({T.edges[e].block, s, 0});
            for (int e : outs) L.elim_trsm.push_back({T.edges[e].block, s, 1});
            if (!lu) {
                // schur_symmetric (tree.cpp:862-883)
                for (int e1 : outs)
                    for (int e2 : outs)
                        if (T.edges[e1].n2 >= T.edges[e2].n2) gemm_edges(e1, e2, false, true);
                for (int e1 : ins)
                    for (int e2 : ins)
                        if (T.edges[e1].n1 >= T.edges[e2].n1) gemm_edges(e1, e2, true, false);
            }
            // the general path's Schur complement is this product alone (tree.cpp:943-947)
            for (int e1 : outs)
                for (int e2 : ins) gemm_edges(e1, e2, false, false);
            // record (tree.cpp:909-910, 885-892; PLU: 950-956)
            L.op_elim_llt.push_back(s);
            L.op_elim_llt_block.push_back(piv);
            for (int e : T.out_nbr(s)) L.op_gemm.push_back({s, T.edges[e].n2, T.edges[e].block, lu ? 6 : 1});
            for (int e : T.in_nbr(s)) L.op_gemm.push_back({s, T.edges[e].n1, T.edges[e].block, lu ? 7 : 2});
            T.set_eliminated(s);
        }
        L.fill_len = cursor - L.fill_off;
        L.schur_first = (int)P.schur_targets.size();
        for (size_t i = 0; i < target_order.size(); i++) {
            auto& ups = pending[target_order[i]];
            SchurTarget t;
            t.target = target_order[i];
            t.syrk = target_syrk[i];
            t.first = (int)P.schur_updates.size();
            t.count = (int)ups.size();
            P.schur_updates.insert(P.schur_updates.end(), ups.begin(), ups.end());
            P.schur_targets.push_back(t);
        }
        L.schur_count = (int)P.schur_targets.size() - L.schur_first;

        if (ilvl >= skip) {
            // ---- scale (tree.cpp:796-856, LLT) ----
            L.scaled = true;
            for (int c : bottom) {
                if (H.level[c] <= ilvl) continue;
                int pe = T.pivot(c);
                int piv = T.edges[pe].block;
                L.scale_clusters.push_back(c);
                L.scale_pivots.push_back(piv);
                L.scale_inv.push_back(lu ? T.new_block(c, c, BLK_STORED, cursor) : -1);
                for (int e : T.in_nbr(c)) L.scale_trsm.push_back({T.edges[e].block, c, 0});
                for (int e : T.out_nbr(c)) L.scale_trsm.push_back({T.edges[e].block, c, 1});
                L.op_scale_llt.push_back(c);
                L.op_scale_llt_block.push_back(piv);
                // the new pivot: I, or diag(sign D) on the LDLT path (tree.cpp:830)
                T.edges[pe].block = T.new_block(c, c, ldlt ? BLK_STORED : BLK_IDENTITY, cursor);
                L.scale_newpiv.push_back(ldlt ? T.edges[pe].block : -1);
            }
            // ---- sparsify (tree.cpp:1417-1433, 1292-1347), scheduled in waves ----
            std::vector<int> wave_of(nc, -1);
            for (int c : bottom) {
                if (H.level[c] <= ilvl) continue;
                if (use_want_sparsify && !H.sparsify[c]) {
                    L.ignored++;
                    continue;
                }
                SparsifyItem it;
                it.cluster = c;
                it.first = (int)P.asn_pieces.size();
                int w = 0;
                int cap_cols = 0;
                for (int e : T.in_nbr(c)) {
                    int n = T.edges[e].n1;
                    P.asn_pieces.push_back({T.edges[e].block, n, 0});
                    cap_cols += P.c_cap[n];
                    if (wave_of[n] >= 0) w = std::max(w, wave_of[n] + 1);
                }
                for (int e : T.out_nbr(c)) {
                    int n = T.edges[e].n2;
                    P.asn_pieces.push_back({T.edges[e].block, n, 1});
                    cap_cols += P.c_cap[n];
                    if (wave_of[n] >= 0) w = std::max(w, wave_of[n] + 1);
                }
                it.count = (int)P.asn_pieces.size() - it.first;
                it.cap_cols = cap_cols;
                it.v_off = P.v_len;
                P.v_len += (int64_t)P.c_cap[c] * P.c_cap[c];
                it.tau_off = P.tau_len;
                P.tau_len += P.c_cap[c];
                if (ldlt) {
                    // sibling: capacity of the cluster, its own solve slot, pivot and edge blocks
                    const int sib = (int)P.c_cap.size();
                    P.c_start.push_back(P.c_start[c]);
                    P.c_cap.push_back(P.c_cap[c]);
                    P.c_level.push_back(P.c_level[c]);
                    P.c_order.push_back(sib);
                    P.c_hlevel.push_back(ilvl);
                    P.c_parent.push_back(-1);
                    P.c_sparsify.push_back(0);
                    P.c_children.push_back({});
                    P.c_xoff.push_back(P.x_len);
                    P.x_len += P.c_cap[c];
                    it.piv = T.edges[T.pivot(c)].block;
                    it.sib = sib;
                    it.sib_piv = T.new_block(sib, sib, BLK_STORED, cursor);
                    it.aso = T.new_block(sib, c, BLK_STORED, cursor);
                }
                wave_of[c] = w;
                if ((int)L.waves.size() <= w) L.waves.resize(w + 1);
                L.waves[w].push_back(it);
                L.op_ortho.push_back(c);
            }
            for (auto& wave : L.waves) {
                int64_t ws = 0;
                for (auto& it : wave) {
                    it.ws_off = ws;
                    ws += (int64_t)P.c_cap[it.cluster] * std::max(it.cap_cols, 1);
                    ws = (ws + 31) & ~int64_t(31);
                }
                L.ws_len = std::max(L.ws_len, ws);
            }
            P.ws_len = std::max(P.ws_len, L.ws_len);
        }

        // ---- merge (tree.cpp:1435-1445, 1106-1184) ----
        if (ilvl < nl - 1) {
            L.merged = true;
            L.merge_off = cursor;
            const std::vector<int>& parents = H.bottoms[ilvl + 1];
            for (int snew : parents) L.op_merge.push_back(snew);
            L.merge_parents = parents;
            for (int snew : parents) {
                std::set<int> nnews;
                for (int sold : H.children[snew])
                    for (int e : T.out[sold]) nnews.insert(H.parent[T.edges[e].n2]);
                for (int nnew : nnews) {
                    int b = T.new_block(nnew, snew, BLK_STORED, cursor);
                    T.add_edge(snew, nnew, b);
                    P.n_merge_blocks++;
                }
                T.sort_edges(snew);
                for (int sold : H.children[snew]) {
                    for (int e : T.out[sold]) {
                        int nold = T.edges[e].n2;
                        int nnew = H.parent[nold];
                        int dst = -1;
                        for (int f : T.out[snew])
                            if (T.edges[f].n2 == nnew) { dst = T.edges[f].block; break; }
                        L.merge_copies.push_back({T.edges[e].block, dst, nold, sold});
                    }
                    T.out[sold].clear();
                    T.in[sold].clear();
                }
            }
            L.merge_len = cursor - L.merge_off;
        }
    }
    P.arena_len = cursor;
    P.nclusters_h = nc;
    P.nclusters = (int)P.c_cap.size();  // with the LDLT siblings
    return P;
}

// tree.cpp:1553-1608 for SPD / LLT.  Per level, every cluster in list order: scale
// (tree.cpp:796-811), then sparsify over its fill-in edges (tree.cpp:1292-1347 with pred =
// !original, 1411-1415): the QRCP's edges take R P^T, the original edges get Q^T and hand
// their last rows to a sibling edge (tree.cpp:1018-1064), and the sibling (identity pivot)
// is eliminated at once, updating its neighbours (tree.cpp:895-910).  The sibling is
// planned whatever the rank; a rank equal to the size gives it no rows, and the fill-in
// blocks it would have created stay zero (the reference creates none: only extra zero
// columns of later QRCP matrices, which never change a rank for tol > 0).  Clusters of a
// level are scheduled in waves (each after every neighbour processed before it, fill-in
// included); every wave is one level of the plan.  Capacities: a cluster's size after its
// sparsification is at most min(its size, the size of its fill-in columns), so a parent's
// capacity is the sum of its children's bounds after their sparsification, and every block
// is allocated with the capacities its clusters have when it is created (they only shrink
// afterwards within the level).
Plan build_plan_lorasp(const Hierarchy& H, const Assembly& asmb) {
    Plan P;
    P.lorasp = true;
    const int nl = H.nlevels;
    const int nc = (int)H.start.size();
    P.nclusters = nc;
    P.c_start = H.start;
    P.c_cap = H.size;
    P.c_level = H.level;
    P.c_hlevel = H.hlevel;
    P.c_parent = H.parent;
    P.c_sparsify = H.sparsify;
    P.c_children = H.children;
    P.c_order.resize(nc);
    std::iota(P.c_order.begin(), P.c_order.end(), 0);
    // solve slots: the leaves now, every parent at its merge (its capacity is known then)
    P.c_xoff.assign(nc, 0);
    for (int c : H.bottoms[0]) {
        P.c_xoff[c] = P.x_len;
        P.x_len += H.size[c];
    }
    std::vector<int> capnow(P.c_cap);  // current capacity bound of every cluster
    SymTree T(H, P);
    int64_t cursor = 0;
    for (size_t li = 0; li < H.bottoms[0].size(); li++) {
        int self = H.bottoms[0][li];
        for (int nbr : asmb.nbrs[li]) {
            int b = T.new_block(nbr, self, BLK_STORED, cursor);
            P.initial_blocks.push_back(b);
            T.add_edge(self, nbr, b, true);
        }
        T.sort_edges(self);
    }
    P.assembled_len = cursor;
    P.lr_order.resize(nl);
    std::vector<int> wave_of;  // per cluster, this level
    for (int ilvl = 0; ilvl < nl; ilvl++) {
        const std::vector<int>& bottom = H.bottoms[ilvl];
        const size_t first = P.levels.size();
        wave_of.assign(P.c_cap.size(), -1);
        // per wave: Schur updates of its siblings, by target in first-touch order
        std::vector<std::map<int, std::vector<SchurUpdate>>> pending;
        std::vector<std::vector<int>> target_order, target_syrk;
        auto level_of = [&](int w) -> LevelPlan& {
            while ((int)(P.levels.size() - first) <= w) {
                P.levels.emplace_back();
                LevelPlan& L = P.levels.back();
                L.real = ilvl;
                L.scaled = true;
                L.waves.resize(1);
                pending.emplace_back();
                target_order.emplace_back();
                target_syrk.emplace_back();
            }
            return P.levels[first + w];
        };
        for (int c : bottom) {
            int w = 0;
            for (int e : T.out[c])
                if (T.edges[e].n2 != c && wave_of[T.edges[e].n2] >= 0) w = std::max(w, wave_of[T.edges[e].n2] + 1);
            for (int e : T.in[c])
                if (wave_of[T.edges[e].n1] >= 0) w = std::max(w, wave_of[T.edges[e].n1] + 1);
            LevelPlan& L = level_of(w);
            // ---- scale (tree.cpp:796-811) ----
            const int pe = T.pivot(c);
            const int piv = T.edges[pe].block;
            L.scale_clusters.push_back(c);
            L.scale_pivots.push_back(piv);
            L.scale_inv.push_back(-1);
            for (int e : T.in_nbr(c)) L.scale_trsm.push_back({T.edges[e].block, c, 0});
            for (int e : T.out_nbr(c)) L.scale_trsm.push_back({T.edges[e].block, c, 1});
            L.op_scale_llt.push_back(c);
            L.op_scale_llt_block.push_back(piv);
            // the new pivot is a stored identity: siblings eliminated later in the level
            // update it (their neighbours' pivots take A^T A)
            T.edges[pe].block = T.new_block(c, c, BLK_STORED, cursor, capnow[c], capnow[c]);
            L.scale_newpiv.push_back(T.edges[pe].block);
            L.snap.push_back(c);
            // ---- sparsify over the fill-in edges ----
            SparsifyItem it;
            it.cluster = c;
            it.first = (int)P.asn_pieces.size();
            int cap_cols = 0;
            const auto ins = T.in_nbr(c);
            const auto outs = T.out_nbr(c);
            for (int e : ins)
                if (!T.orig[e]) {
                    P.asn_pieces.push_back({T.edges[e].block, T.edges[e].n1, 0});
                    cap_cols += capnow[T.edges[e].n1];
                }
            for (int e : outs)
                if (!T.orig[e]) {
                    P.asn_pieces.push_back({T.edges[e].block, T.edges[e].n2, 1});
                    cap_cols += capnow[T.edges[e].n2];
                }
            it.count = (int)P.asn_pieces.size() - it.first;
            it.cap_cols = cap_cols;
            it.v_off = P.v_len;
            P.v_len += (int64_t)P.c_cap[c] * P.c_cap[c];
            it.tau_off = P.tau_len;
            P.tau_len += P.c_cap[c];
            // the sibling: capacity of the cluster, its own solve slot and edge blocks
            const int sib = (int)P.c_cap.size();
            P.c_start.push_back(P.c_start[c]);
            P.c_cap.push_back(P.c_cap[c]);
            P.c_level.push_back(P.c_level[c]);
            P.c_order.push_back(sib);
            P.c_hlevel.push_back(ilvl);
            P.c_parent.push_back(-1);
            P.c_sparsify.push_back(0);
            P.c_children.push_back({});
            P.c_xoff.push_back(P.x_len);
            P.x_len += P.c_cap[c];
            T.out.emplace_back();
            T.in.emplace_back();
            T.eliminated.push_back(0);
            wave_of.push_back(-1);
            capnow.push_back(capnow[c]);
            it.sib = sib;
            T.add_edge(sib, sib, T.new_block(sib, sib, BLK_IDENTITY, cursor), true);
            it.ofirst = (int)P.lr_splits.size();
            auto split = [&](int e, int n, int tr) {
                const int sb = T.new_block(sib, n, BLK_STORED, cursor, capnow[sib], capnow[n]);
                P.lr_splits.push_back({T.edges[e].block, n, tr, sb});
                T.add_edge(n, sib, sb, true);
            };
            for (int e : ins)
                if (T.orig[e]) split(e, T.edges[e].n1, 0);
            for (int e : outs)
                if (T.orig[e]) split(e, T.edges[e].n2, 1);
            it.ocount = (int)P.lr_splits.size() - it.ofirst;
            // ---- eliminate the sibling (tree.cpp:895-910): identity pivot, Schur updates
            // between the neighbours of its original edges (tree.cpp:862-883) ----
            auto& pend = pending[w];
            const auto sins = T.in_nbr(sib);
            for (int e1 : sins)
                for (int e2 : sins) {
                    const int n1 = T.edges[e1].n1, n2 = T.edges[e2].n1;
                    if (n1 < n2) continue;
                    int found = -1;
                    for (int e : T.out[n2])
                        if (T.edges[e].n2 == n1) { found = e; break; }
                    if (found < 0) {
                        found = T.add_edge(n2, n1, T.new_block(n1, n2, BLK_STORED, cursor, capnow[n1], capnow[n2]),
                                           false);
                        P.n_fill_blocks++;
                    }
                    const int tb = T.edges[found].block;
                    auto pt = pend.find(tb);
                    if (pt == pend.end()) {
                        target_order[w].push_back(tb);
                        target_syrk[w].push_back(n1 == n2 ? 1 : 0);
                        pt = pend.emplace(tb, std::vector<SchurUpdate>()).first;
                    }
                    pt->second.push_back({T.edges[e1].block, 1, T.edges[e2].block, 0, sib});
                }
            it.sfirst = (int)P.lr_sibops.size();
            for (int e : sins) {
                const int n = T.edges[e].n1;
                P.lr_sibops.push_back({n, T.edges[e].block, wave_of[n] >= 0 ? 1 : 0});
            }
            it.scount = (int)P.lr_sibops.size() - it.sfirst;
            T.set_eliminated(sib);
            capnow[c] = std::min(capnow[c], cap_cols);  // rank <= min(rows, fill-in columns)
            wave_of[c] = w;
            P.lr_order[ilvl].push_back({c, (int)(first + w), (int)L.waves[0].size()});
            L.waves[0].push_back(it);
            L.op_ortho.push_back(c);
        }
        // per plan level: the workspace of its wave and its Schur targets
        for (size_t w = 0; first + w < P.levels.size(); w++) {
            LevelPlan& L = P.levels[first + w];
            int64_t ws = 0;
            for (auto& it : L.waves[0]) {
                it.ws_off = ws;
                ws += (int64_t)P.c_cap[it.cluster] * std::max(it.cap_cols, 1);
                ws = (ws + 31) & ~int64_t(31);
            }
            L.ws_len = ws;
            P.ws_len = std::max(P.ws_len, ws);
            L.schur_first = (int)P.schur_targets.size();
            for (size_t i = 0; i < target_order[w].size(); i++) {
                auto& ups = pending[w][target_order[w][i]];
                P.schur_targets.push_back({target_order[w][i], target_syrk[w][i], (int)P.schur_updates.size(),
                                           (int)ups.size()});
                P.schur_updates.insert(P.schur_updates.end(), ups.begin(), ups.end());
            }
            L.schur_count = (int)P.schur_targets.size() - L.schur_first;
        }
        if (P.levels.size() == first) level_of(0);  // an empty level still merges
        // ---- merge (tree.cpp:1106-1184): an edge between parents is original when one of
        // the edges it gathers is ----
        if (ilvl < nl - 1) {
            LevelPlan& L = P.levels.back();
            L.merged = true;
            L.merge_off = cursor;
            const std::vector<int>& parents = H.bottoms[ilvl + 1];
            for (int snew : parents) L.op_merge.push_back(snew);
            L.merge_parents = parents;
            for (int snew : parents) {  // capacity: the children's bounds after this level
                int cap = 0;
                for (int sold : H.children[snew]) cap += capnow[sold];
                P.c_cap[snew] = capnow[snew] = cap;
                P.c_xoff[snew] = P.x_len;
                P.x_len += cap;
            }
            for (int snew : parents) {
                std::map<int, char> nnews;
                for (int sold : H.children[snew])
                    for (int e : T.out[sold]) nnews[H.parent[T.edges[e].n2]] |= T.orig[e];
                for (const auto& kv : nnews) {
                    int b = T.new_block(kv.first, snew, BLK_STORED, cursor);
                    T.add_edge(snew, kv.first, b, kv.second != 0);
                    P.n_merge_blocks++;
                }
                T.sort_edges(snew);
                for (int sold : H.children[snew]) {
                    for (int e : T.out[sold]) {
                        int nold = T.edges[e].n2;
                        int nnew = H.parent[nold];
                        int dst = -1;
                        for (int f : T.out[snew])
                            if (T.edges[f].n2 == nnew) { dst = T.edges[f].block; break; }
                        L.merge_copies.push_back({T.edges[e].block, dst, nold, sold});
                    }
                    T.out[sold].clear();
                    T.in[sold].clear();
                }
            }
            L.merge_len = cursor - L.merge_off;
        }
    }
    P.nlevels = (int)P.levels.size();
    P.arena_len = cursor;
    P.nclusters_h = nc;
    P.nclusters = (int)P.c_cap.size();
    return P;
}

std::vector<int64_t> assembly_map(const Plan& P, const Hierarchy& H, const Assembly& asmb, const Csc& A,
                                  const std::vector<int>& perm) {
    const int N = A.n;
    std::vector<int> pinv(N), owner(N);
    for (int i = 0; i < N; i++) pinv[perm[i]] = i;
    for (int c : H.bottoms[0])
        for (int k = H.start[c]; k < H.start[c] + H.size[c]; k++) owner[k] = c;
    // per leaf: (neighbour, block) in the order assembly created them (self first, then by order)
    std::vector<int> leaf_index(H.start.size(), -1);
    for (size_t li = 0; li < H.bottoms[0].size(); li++) leaf_index[H.bottoms[0][li]] = (int)li;
    std::vector<size_t> first(H.bottoms[0].size() + 1, 0);
    for (size_t li = 0; li < H.bottoms[0].size(); li++) first[li + 1] = first[li] + asmb.nbrs[li].size();
    std::vector<int64_t> map(A.rowval.size(), -1);
    for (int col = 0; col < N; col++) {
        const int j = pinv[col];
        const int self = owner[j];
        const int li = leaf_index[self];
        const std::vector<int>& nb = asmb.nbrs[li];
        for (int k = A.colptr[col]; k < A.colptr[col + 1]; k++) {
            const int i = pinv[A.rowval[k]];
            const int nbr = owner[i];
            int t = -1;
            if (nbr == self) {
                t = 0;
            } else {
                auto it = std::lower_bound(nb.begin() + 1, nb.end(), nbr);
                if (it != nb.end() && *it == nbr) t = (int)(it - nb.begin());
            }
            if (t < 0) continue;
            const PlanBlock& B = P.blocks[P.initial_blocks[first[li] + t]];
            map[k] = B.off + (int64_t)(i - H.start[nbr]) + (int64_t)(j - H.start[self]) * B.ld;
        }
    }
    return map;
}

}  // namespace spand

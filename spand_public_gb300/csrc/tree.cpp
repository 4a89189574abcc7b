// spaND::Tree on the GB300 device path.  Citations are path:line into
// leopoldcambier/spaND_public.
#include "tree.h"

#include <chrono>
#include <cmath>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <numeric>

namespace spaND {

static double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

static void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

void upload_csr(const Csc& A, spand::DeviceCsr& dA, int** d_cmap) {
    const int n = A.n;
    const size_t nnz = A.rowval.size();
    std::vector<int> rp(n + 1, 0), ci(nnz), cmap(nnz);
    for (int j = 0; j < n; j++)
        for (int k = A.colptr[j]; k < A.colptr[j + 1]; k++) rp[A.rowval[k] + 1]++;
    for (int i = 0; i < n; i++) rp[i + 1] += rp[i];
    std::vector<int> fill(rp.begin(), rp.end() - 1);
    for (int j = 0; j < n; j++)
        for (int k = A.colptr[j]; k < A.colptr[j + 1]; k++) {
            const int r = A.rowval[k];
            ci[fill[r]] = j;
            cmap[k] = fill[r]++;
        }
    if (dA.rowptr) { cudaFree(dA.rowptr); cudaFree(dA.colind); cudaFree(dA.val); }
    if (*d_cmap) cudaFree(*d_cmap);
    dA.n = n;
    cuda_check(cudaMalloc(&dA.rowptr, rp.size() * sizeof(int)), "cudaMalloc");
    cuda_check(cudaMalloc(&dA.colind, std::max<size_t>(nnz, 1) * sizeof(int)), "cudaMalloc");
    cuda_check(cudaMalloc(&dA.val, std::max<size_t>(nnz, 1) * sizeof(double)), "cudaMalloc");
    cuda_check(cudaMalloc(d_cmap, std::max<size_t>(nnz, 1) * sizeof(int)), "cudaMalloc");
    cuda_check(cudaMemcpy(dA.rowptr, rp.data(), rp.size() * sizeof(int), cudaMemcpyHostToDevice), "H2D");
    cuda_check(cudaMemcpy(dA.colind, ci.data(), nnz * sizeof(int), cudaMemcpyHostToDevice), "H2D");
    cuda_check(cudaMemcpy(*d_cmap, cmap.data(), nnz * sizeof(int), cudaMemcpyHostToDevice), "H2D");
}

Tree::Tree(int nlevels) : nlevels_(nlevels) {
    if (nlevels <= 0) throw std::invalid_argument("nlevels must be > 0");  // tree.cpp:87
}

double* Tree::cg_buffer(int which, int n) const {
    spand::DeviceScope scope(device_);
    if (cg_len_ < (size_t)n) {
        for (auto& p : cg_buf_)
            if (p) cudaFree(p);
        cg_buf_[0] = cg_buf_[1] = nullptr;
        cuda_check(cudaMalloc(&cg_buf_[0], n * sizeof(double)), "cudaMalloc");
        cuda_check(cudaMalloc(&cg_buf_[1], n * sizeof(double)), "cudaMalloc");
        cg_len_ = n;
    }
    return cg_buf_[which];
}

Tree::~Tree() {
    spand::DeviceScope scope(device_);
    dev_.reset();
    for (auto& p : cg_buf_)
        if (p) cudaFree(p);
    if (d_cmap_) cudaFree(d_cmap_);
    if (d_prow_) cudaFree(d_prow_);
    if (d_pcol_) cudaFree(d_pcol_);
    if (dx_) cudaFree(dx_);
    if (dA_.rowptr) cudaFree(dA_.rowptr);
    if (dA_.colind) cudaFree(dA_.colind);
    if (dA_.val) cudaFree(dA_.val);
    if (stream_) cudaStreamDestroy(stream_);
}

void Tree::set_Xcoo(const double* X, int dim, int n) {
    X_.assign(X, X + (size_t)dim * n);
    dim_ = dim;
}

// tree.cpp:306-419
std::vector<ClusterID> Tree::partition(const Csc& A) {
    if (partitioned_) throw std::logic_error("partition() called twice");
    double t0 = now_s();
    const int N = A.n;
    if (part_kind_ != PartKind::MND) throw std::invalid_argument("only modified nested dissection (MND) is supported");
    if (geo_) {
        if ((int)X_.size() != dim_ * N || dim_ <= 0) throw std::invalid_argument("set_Xcoo: coordinates must be dim x N");
        part_ = spand::partition_modified_nd(A, nlevels_, X_.data(), dim_);
    } else {
        std::string err;
        if (!spand::partition_modified_nd_metis(A, nlevels_, part_, err)) throw std::runtime_error(err);
    }
    H_ = spand::build_hierarchy(part_, nlevels_, perm_);
    log_.assign(nlevels_, LevelLog());
    for (int i = 0; i < N; i++) log_[part_[i].self.lvl].dofs_nd += 1;
    log_[nlevels_ - 1].dofs_left_nd = 0;
    for (int l = nlevels_ - 2; l >= 0; l--) log_[l].dofs_left_nd = log_[l + 1].dofs_nd + log_[l + 1].dofs_left_nd;
    partitioned_ = true;
    t_partition = now_s() - t0;
    return part_;
}

std::vector<int> Tree::partition_lorasp(const Csc& A) {
    if (partitioned_) throw std::logic_error("partition() called twice");
    double t0 = now_s();
    const int N = A.n;
    if (!geo_) throw std::invalid_argument("LoRaSp ordering needs coordinates (set_Xcoo, set_use_geo)");
    if ((int)X_.size() != dim_ * N || dim_ <= 0) throw std::invalid_argument("set_Xcoo: coordinates must be dim x N");
    std::vector<int> parts = spand::partition_rb(N, nlevels_, X_.data(), dim_);
    H_ = spand::build_hierarchy_lorasp(parts, nlevels_, perm_);
    log_.assign(nlevels_, LevelLog());
    part_.clear();
    lorasp_ = true;
    partitioned_ = true;
    t_partition = now_s() - t0;
    return parts;
}

void Tree::factorize_lorasp() {
    if (!lorasp_) throw std::logic_error("factorize_lorasp() needs partition_lorasp()");
    lorasp_run_ = true;
    factorize();
}

// tree.cpp:505-575, plus the symbolic plan of factorize() and the device upload.  The
// block values are assembled on the device: the first call builds the map from every
// entry of A to its place in the level-0 blocks; later calls with the same sparsity
// pattern only copy the new values and scatter them.
void Tree::assemble(const Csc& A) {
    if (!partitioned_) throw std::logic_error("assemble() before partition()");
    spand::DeviceScope scope(device_);
    const bool lu = symm_ == SymmKind::GEN;
    const bool ldlt = symm_ == SymmKind::SYM;
    if (!((symm_ == SymmKind::SPD && scaling_ == ScalingKind::LLT) || (lu && scaling_ == ScalingKind::PLU) ||
          (ldlt && scaling_ == ScalingKind::LDLT)))
        throw std::invalid_argument("the device path implements the SPD / LLT, SYM / LDLT and GEN / PLU configurations");
    if (A.n != get_N()) throw std::invalid_argument("matrix size does not match the partition");
    if ((int64_t)A.val.size() != (int64_t)A.rowval.size()) throw std::invalid_argument("values do not match the pattern");
    double t0 = now_s();
    const bool same_pattern = assembled_ok_ && dev_ && A.colptr == A_.colptr && A.rowval == A_.rowval;
    if (!same_pattern) {
        A_ = A;
        Csc App = spand::symm_perm(A, perm_);
        asmb_ = spand::assembly_structure(H_, App, !lu);
        if (lorasp_) {
            if (symm_ != SymmKind::SPD) throw std::invalid_argument("LoRaSp is implemented for SPD / LLT");
            plan_ = spand::build_plan_lorasp(H_, asmb_);
        } else {
            plan_ = spand::build_plan(H_, asmb_, skip_, use_want_sparsify_, lu, ldlt);
        }
        std::vector<int64_t> amap = spand::assembly_map(plan_, H_, asmb_, A, perm_);
        if (!stream_) {
            // the tree lives on the device current at its first assembly
            device_ = spand::current_device();
            cuda_check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
        }
        dev_ = spand::make_device_factor(fp32_, stream_, perm_);
        try {
            dev_->upload(plan_, amap);
        } catch (spand::DeviceError& e) {
            throw std::runtime_error(e.msg);
        }
        if (d_prow_) cudaFree(d_prow_);
        if (d_pcol_) cudaFree(d_pcol_);
        d_prow_ = d_pcol_ = nullptr;
        upload_csr(A, dA_, &d_cmap_);
    } else {
        A_.val = A.val;
    }
    try {
        dev_->assemble_values(A.val.data(), (int64_t)A.val.size());
    } catch (spand::DeviceError& e) {
        throw std::runtime_error(e.msg);
    }
    spand::device_scatter(dev_->device_values(), d_cmap_, (int64_t)A.val.size(), dA_.val, stream_);
    cuda_check(cudaGetLastError(), "assembly scatter");
    cuda_check(cudaStreamSynchronize(stream_), "sync");
    assembled_ok_ = true;
    factored_ = false;
    t_assemble = now_s() - t0;
}

bool Tree::assemble_same_pattern(int n, const int* colptr, const int* rowval, const double* vals) {
    spand::DeviceScope scope(device_);
    if (!assembled_ok_ || !dev_ || n != A_.n || !colptr || !vals) return false;
    if (std::memcmp(colptr, A_.colptr.data(), ((size_t)n + 1) * sizeof(int)) != 0) return false;
    const size_t nnz = A_.rowval.size();
    if (nnz && (!rowval || std::memcmp(rowval, A_.rowval.data(), nnz * sizeof(int)) != 0)) return false;
    double t0 = now_s();
    std::memcpy(A_.val.data(), vals, nnz * sizeof(double));
    try {
        dev_->assemble_values(vals, (int64_t)nnz);
    } catch (spand::DeviceError& e) {
        throw std::runtime_error(e.msg);
    }
    spand::device_scatter(dev_->device_values(), d_cmap_, (int64_t)nnz, dA_.val, stream_);
    cuda_check(cudaGetLastError(), "assembly scatter");
    cuda_check(cudaStreamSynchronize(stream_), "sync");
    factored_ = false;
    t_assemble = now_s() - t0;
    return true;
}

void Tree::assemble_values(const double* vals, int64_t nnz, bool on_device) {
    spand::DeviceScope scope(device_);
    if (!assembled_ok_ || !dev_) throw std::logic_error("assemble_values() before assemble()");
    if (nnz != (int64_t)A_.rowval.size()) throw std::invalid_argument("values do not match the assembled pattern");
    double t0 = now_s();
    if (!on_device) A_.val.assign(vals, vals + nnz);
    try {
        dev_->assemble_values(vals, nnz, on_device);
    } catch (spand::DeviceError& e) {
        throw std::runtime_error(e.msg);
    }
    spand::device_scatter(dev_->device_values(), d_cmap_, nnz, dA_.val, stream_);
    cuda_check(cudaGetLastError(), "assembly scatter");
    cuda_check(cudaStreamSynchronize(stream_), "sync");
    factored_ = false;
    t_assemble = now_s() - t0;
}

// The reference's message for a failed pivot: tree.cpp:587-590 (LLT), 624-628 (PLU)
std::string Tree::pivot_error() const {
    return symm_ == SymmKind::GEN ? "Error: Singular Pivot\n" : "Error: Non-SPD Pivot\n";
}

void Tree::set_phi(const double* phi, int n, int nphi) {
    if (n < 0 || nphi < 0 || (n * (long long)nphi > 0 && !phi)) throw std::invalid_argument("bad phi");
    phi_.assign(phi, phi + (size_t)n * nphi);
    phi_n_ = n;
    nphi_ = nphi;
}

// tree.cpp:1457-1459, 1477-1485: preservation needs a symmetric kind and phi of N rows
void Tree::prepare_factorize() {
    if (!assembled_ok_) throw std::logic_error("factorize() before assemble()");
    if (lorasp_ && !lorasp_run_)
        throw std::logic_error("a tree partitioned with partition_lorasp() factorizes with factorize_lorasp()");
    lorasp_run_ = false;
    if (lorasp_ && preserve_) throw std::invalid_argument("LoRaSp does not preserve vectors (tree.cpp:1564)");
    try {
        if (!preserve_) {
            dev_->set_phi(nullptr, 0, 0);
            return;
        }
        if (symm_ == SymmKind::GEN) throw std::invalid_argument("preservation needs a symmetric matrix (SPD or SYM)");
        if (nphi_ <= 0 || phi_n_ != get_N()) throw std::invalid_argument("preservation needs phi with N rows");
        dev_->set_phi(phi_.data(), phi_n_, nphi_);
    } catch (spand::DeviceError& e) {
        throw std::runtime_error(e.msg);
    }
}

// tree.cpp:1447-1551
void Tree::factorize() {
    spand::DeviceScope scope(device_);
    prepare_factorize();
    double t0 = now_s();
    try {
        dev_->factorize(tol_);
    } catch (spand::DeviceError& e) {
        if (e.status == spand::SPAND_ERR_NOT_SPD) {
            if (verb_) printf(symm_ == SymmKind::GEN ? "Singular Pivot!\n" : "Not SPD!\n");
            throw std::runtime_error(pivot_error());
        }
        throw std::runtime_error(e.msg);
    }
    t_factorize = now_s() - t0;
    factored_ = true;
    log_dirty_ = true;
}

void Tree::factorize_enqueue() {
    spand::DeviceScope scope(device_);
    prepare_factorize();
    try {
        dev_->factorize_enqueue(tol_);
    } catch (spand::DeviceError& e) {
        throw std::runtime_error(e.msg);
    }
}

void Tree::factorize_finish() {
    spand::DeviceScope scope(device_);
    try {
        dev_->factorize_finish();
    } catch (spand::DeviceError& e) {
        if (e.status == spand::SPAND_ERR_NOT_SPD) {
            if (verb_) printf(symm_ == SymmKind::GEN ? "Singular Pivot!\n" : "Not SPD!\n");
            throw std::runtime_error(pivot_error());
        }
        throw std::runtime_error(e.msg);
    }
    factored_ = true;
    log_dirty_ = true;
}

spand::PcgWork& Tree::pcg_work() const {
    if (!pcg_work_) pcg_work_.reset(new spand::PcgWork());
    return *pcg_work_;
}

void Tree::bench_step(const double* b_dev, double* x_dev, int nrhs, int iters, double tol, double out[4]) {
    spand::DeviceScope scope(device_);
    prepare_factorize();
    cudaEvent_t e[3];
    for (auto& ev : e) cuda_check(cudaEventCreate(&ev), "cudaEventCreate");
    spand::PcgResult r;
    try {
        cuda_check(cudaEventRecord(e[0], stream_), "cudaEventRecord");
        dev_->factorize(tol_);
        factored_ = true;
        log_dirty_ = true;
        cuda_check(cudaEventRecord(e[1], stream_), "cudaEventRecord");
        cuda_check(cudaMemsetAsync(x_dev, 0, (size_t)get_N() * nrhs * sizeof(double), stream_), "cudaMemsetAsync");
        if (nrhs == 1) {
            r = spand::device_pcg(*dev_, dA_, b_dev, x_dev, iters, tol, true);
        } else {
            std::vector<int> its(nrhs);
            std::vector<double> rel(nrhs);
            spand::device_pcg_multi(*dev_, dA_, b_dev, x_dev, nrhs, iters, tol, true, its.data(), rel.data());
            r.iterations = *std::max_element(its.begin(), its.end());
            r.relres = *std::max_element(rel.begin(), rel.end());
        }
        cuda_check(cudaEventRecord(e[2], stream_), "cudaEventRecord");
        cuda_check(cudaEventSynchronize(e[2]), "cudaEventSynchronize");
    } catch (spand::DeviceError& err) {
        for (auto& ev : e) cudaEventDestroy(ev);
        if (err.status == spand::SPAND_ERR_NOT_SPD) throw std::runtime_error(pivot_error());
        throw std::runtime_error(err.msg);
    }
    float f = 0, p = 0;
    cudaEventElapsedTime(&f, e[0], e[1]);
    cudaEventElapsedTime(&p, e[1], e[2]);
    for (auto& ev : e) cudaEventDestroy(ev);
    out[0] = f;
    out[1] = p;
    out[2] = r.iterations;
    out[3] = r.relres;
}

void Tree::solve_device(double* x, int nrhs, int ld) const {
    spand::DeviceScope scope(device_);
    if (!factored_) throw std::logic_error("solve() before factorize()");
    try {
        dev_->solve_device(x, nrhs, ld);
    } catch (spand::DeviceError& e) {
        throw std::runtime_error(e.msg);
    }
}

void Tree::solve_device_noalloc(double* x, int nrhs, int ld) const {
    spand::DeviceScope scope(device_);
    if (!factored_) throw std::logic_error("solve() before factorize()");
    try {
        dev_->solve_device_noalloc(x, nrhs, ld);
    } catch (spand::DeviceError& e) {
        if (e.status == spand::SPAND_ERR_ARG) throw std::invalid_argument(e.msg);
        if (e.status == spand::SPAND_ERR_STATE) throw std::logic_error(e.msg);
        throw std::runtime_error(e.msg);
    }
}

void Tree::solve(double* x, int nrhs, int ld) const {
    spand::DeviceScope scope(device_);
    if (ld < 0) ld = get_N();
    const size_t len = (size_t)ld * nrhs;
    if (dx_len_ < len) {
        if (dx_) cudaFree(dx_);
        cuda_check(cudaMalloc(&dx_, len * sizeof(double)), "cudaMalloc");
        dx_len_ = len;
    }
    cuda_check(cudaMemcpyAsync(dx_, x, len * sizeof(double), cudaMemcpyHostToDevice, stream_), "H2D");
    solve_device(dx_, nrhs, ld);
    cuda_check(cudaMemcpyAsync(x, dx_, len * sizeof(double), cudaMemcpyDeviceToHost, stream_), "D2H");
    cuda_check(cudaStreamSynchronize(stream_), "sync");
}

size_t Tree::device_bytes() const { return dev_ ? dev_->device_bytes() : 0; }

// Op list and per-level log reconstructed from the plan and the device sizes, in the
// reference's recording order (tree.cpp:909-910, 885-892, 810, 1331, 1102, 1342, 1439).
// The op list and per-level log of factorize_lorasp, in the reference's order: per cluster
// ScalingLLT, then (rank < size) Orthogonal, Split, the sibling's ScalingLLT (identity)
// and its GemmSymmIn ops; the level's Merge ops at its end.
void Tree::build_ops_and_log_lorasp() {
    spand::DeviceScope scope(device_);
    const spand::Plan& P = plan_;
    long long nnz = 0;
    auto push = [&](OpRecord r) {
        switch (r.kind) {  // Operation::nnz (operations.h:32-163)
            case 0: nnz += (long long)r.ns * (r.ns + 1) / 2; break;
            case 2: nnz += (long long)r.ns * r.nn; break;
            case 3: nnz += (long long)r.ns * r.ns; break;
            default: break;
        }
        ops_.push_back(r);
    };
    std::vector<char> done(P.nclusters, 0);
    int next_order = P.nclusters_h;  // the reference numbers a sibling when it creates one
    for (int rl = 0; rl < (int)P.lr_order.size(); rl++) {
        LevelLog& G = log_[rl];
        for (const auto& rec : P.lr_order[rl]) {
            const int c = rec[0];
            const spand::LevelPlan& L = P.levels[rec[1]];
            const spand::SparsifyItem& it = L.waves[0][rec[2]];
            int blk = -1;
            for (size_t k = 0; k < L.op_scale_llt.size(); k++)
                if (L.op_scale_llt[k] == c) blk = L.op_scale_llt_block[k];
            const int rows = rows0_[c], k = csize_[c];
            push({0, rl, c, -1, rows, 0, rows, rows, blk, c});
            G.rank_before_sum += rows;
            G.rank_after_sum += k;
            G.rank_after_count += 1;
            long long cols = 0;
            for (int p = 0; p < it.count; p++) {
                const int n = P.asn_pieces[it.first + p].nbr;
                cols += done[n] ? csize_[n] : rows0_[n];
            }
            G.nbrs_sum += cols;
            G.nbrs_count += 1;
            if (k < rows) {
                const int sib = next_order++;
                push({3, rl, c, -1, rows, 0, rows, k, c});
                push({5, rl, c, sib, k, rows - k, 0, 0, -1});
                push({0, rl, sib, -1, rows - k, 0, rows - k, rows - k, -1});
                for (int q = 0; q < it.scount; q++) {
                    const spand::LoraSibOp& op = P.lr_sibops[it.sfirst + q];
                    const int nn = op.cur ? csize_[op.nbr] : rows0_[op.nbr];
                    push({2, rl, sib, op.nbr, rows - k, nn, rows - k, nn, op.block});
                }
            }
            done[c] = 1;
        }
        long long left = 0;
        for (const auto& rec : P.lr_order[rl]) left += csize_[rec[0]];
        for (const spand::LevelPlan& L : P.levels)
            if (L.real == rl)
                for (int p : L.op_merge) push({4, rl, p, -1, rows0_[p], 0, 0, 0, -1});
        G.dofs_left_spars = left;
        G.fact_nnz = nnz;
    }
}

void Tree::build_ops_and_log() {
    spand::DeviceScope scope(device_);
    log_dirty_ = false;
    dev_->sizes(csize_, rows0_);
    if (plan_.lorasp) {
        ops_.clear();
        for (LevelLog& G : log_) G = LevelLog();
        build_ops_and_log_lorasp();
        return;
    }
    ops_.clear();
    for (LevelLog& G : log_) {  // keep the partition counts, recompute the rest
        LevelLog fresh;
        fresh.dofs_nd = G.dofs_nd;
        fresh.dofs_left_nd = G.dofs_left_nd;
        G = fresh;
    }
    const spand::Plan& P = plan_;
    int next_order = P.nclusters_h;  // siblings are numbered after all clusters
    long long nnz = 0;
    // pivot ops: ScalingLLT (0), ScalingPLUQ (8) on the general path, ScalingLDLT (9)
    const int kpiv = P.lu ? 8 : P.ldlt ? 9 : 0;
    auto push = [&](OpRecord r) {
        switch (r.kind) {  // Operation::nnz (operations.h:32-163)
            case 0: nnz += (long long)r.ns * (r.ns + 1) / 2; break;
            case 1: case 2: case 6: case 7: nnz += (long long)r.ns * r.nn; break;
            case 3: nnz += (long long)r.ns * r.ns; break;
            case 8: nnz += (long long)r.ns * r.ns + 2LL * r.ns; break;
            case 9: nnz += (long long)r.ns * (r.ns + 1) / 2 + 2LL * r.ns; break;
            default: break;
        }
        ops_.push_back(r);
    };
    for (int l = 0; l < P.nlevels; l++) {
        const spand::LevelPlan& L = P.levels[l];
        LevelLog& G = log_[l];
        size_t g = 0;
        for (size_t k = 0; k < L.op_elim_llt.size(); k++) {
            int s = L.op_elim_llt[k];
            push({kpiv, l, s, -1, rows0_[s], 0, rows0_[s], rows0_[s], L.op_elim_llt_block[k], s});
            while (g < L.op_gemm.size() && L.op_gemm[g].self == s) {
                const spand::GemmOpItem& it = L.op_gemm[g];
                int ns = rows0_[s], nn = rows0_[it.nbr];
                if (it.kind == 1 || it.kind == 6) push({it.kind, l, s, it.nbr, ns, nn, nn, ns, it.block});
                else push({it.kind, l, s, it.nbr, ns, nn, ns, nn, it.block});
                g++;
            }
        }
        long long left_elim = 0;
        for (int c : H_.bottoms[l])
            if (H_.level[c] > l) left_elim += rows0_[c];
        G.dofs_left_elim = left_elim;
        for (size_t k = 0; k < L.op_scale_llt.size(); k++) {
            int c = L.op_scale_llt[k];
            push({kpiv, l, c, -1, rows0_[c], 0, rows0_[c], rows0_[c], L.op_scale_llt_block[k], c});
        }
        // wave index of every sparsified cluster of this level, for the Asn widths
        std::vector<int> wave_of;
        std::map<int, int> wmap;
        for (size_t w = 0; w < L.waves.size(); w++)
            for (const spand::SparsifyItem& it : L.waves[w]) wmap[it.cluster] = (int)w;
        for (int c : L.op_ortho) {
            int rows = rows0_[c], k = csize_[c];
            G.rank_before_sum += rows;
            G.rank_after_sum += k;
            G.rank_after_count += 1;
            // Asn width at this cluster's turn
            const spand::SparsifyItem* item = nullptr;
            for (const auto& wave : L.waves)
                for (const auto& it : wave)
                    if (it.cluster == c) item = &it;
            long long cols = 0;
            for (int p = 0; p < item->count; p++) {
                int n = P.asn_pieces[item->first + p].nbr;
                auto wn = wmap.find(n);
                bool before = wn != wmap.end() && wn->second < wmap[c];
                cols += before ? csize_[n] : rows0_[n];
            }
            if (!(preserve_ && tol_ > 1.0)) {  // preserve-only assembles no Asn (tree.cpp:1257-1287)
                G.nbrs_sum += cols;
                G.nbrs_count += 1;
            }
            if (k < rows) {
                push({3, l, c, -1, rows, 0, rows, k, c});
                int sib = next_order++;
                push({5, l, c, sib, k, rows - k, 0, 0, -1});
                if (P.ldlt) {
                    // the sibling's pivot and its edge to the cluster (tree.cpp:1340-1341)
                    push({9, l, sib, -1, rows - k, 0, rows - k, rows - k, item->sib_piv, item->sib});
                    push({2, l, sib, c, rows - k, k, rows - k, k, item->aso, item->sib});
                } else {
                    push({kpiv, l, sib, -1, rows - k, 0, rows - k, rows - k, -1});
                }
            }
        }
        G.ignored = L.ignored;
        for (int p : L.op_merge) push({4, l, p, -1, rows0_[p], 0, 0, 0, -1});
        long long left_spars = 0;
        if (l + 1 < P.nlevels) {
            for (int p : H_.bottoms[l + 1]) left_spars += rows0_[p];
        }
        G.dofs_left_spars = left_spars;
        G.fact_nnz = nnz;
    }
}

long long Tree::nnz() const {
    ensure_log();
    return log_.empty() ? 0 : log_.back().fact_nnz;
}

// tree.cpp:158-169
int Tree::get_stop() const {
    ensure_log();
    int stop = get_N();
    for (const LevelLog& l : log_) {
        if (l.dofs_left_elim > 0) stop = std::min<long long>(stop, l.dofs_left_elim);
        if (l.dofs_left_spars > 0) stop = std::min<long long>(stop, l.dofs_left_spars);
    }
    return stop;
}

void Tree::print_log() const {
    ensure_log();
    auto mean = [](long long sum, long long count) { return count > 0 ? (double)sum / (double)count : 0.0; };
    printf("spaND factorization log: %d levels, N = %d, tol = %.1e, skip = %d, %s factor\n", nlevels_, get_N(), tol_,
           skip_, fp32_ ? "FP32" : "FP64");
    printf("%5s | %9s %9s %9s %9s | %10s | %9s %9s %9s | %9s %9s %9s %9s\n", "lvl", "nd", "left nd", "left el",
           "left sp", "fact nnz", "rank bfr", "rank aft", "nbrs", "sum bfr", "sum aft", "sparsif", "ignored");
    for (int l = 0; l < (int)log_.size(); l++) {
        const LevelLog& g = log_[l];
        printf("%5d | %9lld %9lld %9lld %9lld | %10.3e | %9.1f %9.1f %9.1f | %9lld %9lld %9lld %9lld\n", l, g.dofs_nd,
               g.dofs_left_nd, g.dofs_left_elim, g.dofs_left_spars, (double)g.fact_nnz,
               mean(g.rank_before_sum, g.rank_after_count), mean(g.rank_after_sum, g.rank_after_count),
               mean(g.nbrs_sum, g.nbrs_count), g.rank_before_sum, g.rank_after_sum, g.rank_after_count, g.ignored);
    }
    printf("stop = %d, factor nnz = %lld, partition %.3e s, assemble %.3e s, factorize %.3e s\n", get_stop(), nnz(),
           t_partition, t_assemble, t_factorize);
}

std::vector<std::array<int, 4>> Tree::ranks() const {
    ensure_log();
    std::vector<std::array<int, 4>> r;
    if (plan_.lorasp) {
        for (int l = 0; l < (int)plan_.lr_order.size(); l++)
            for (const auto& rec : plan_.lr_order[l]) r.push_back({l, rec[0], rows0_[rec[0]], csize_[rec[0]]});
        return r;
    }
    for (int l = 0; l < plan_.nlevels; l++)
        for (int c : plan_.levels[l].op_ortho) r.push_back({l, c, rows0_[c], csize_[c]});
    return r;
}

void Tree::op_matrix(int idx, std::vector<double>& out) const {
    spand::DeviceScope scope(device_);
    const OpRecord& r = ops_.at(idx);
    out.clear();
    if (r.kind == 0 || r.kind == 1 || r.kind == 2 || (r.kind >= 6 && r.kind <= 9)) {
        if (r.block < 0) {  // sibling identity
            out.assign((size_t)r.rows * r.cols, 0.0);
            for (int i = 0; i < r.rows; i++) out[i + (size_t)i * r.rows] = 1.0;
            return;
        }
        std::vector<double> full;
        dev_->block(r.block, full);
        const int ld = plan_.blocks[r.block].ld;
        out.resize((size_t)r.rows * r.cols);
        for (int j = 0; j < r.cols; j++)
            for (int i = 0; i < r.rows; i++) out[i + (size_t)j * r.rows] = full[i + (size_t)j * ld];
    } else if (r.kind == 3) {
        std::vector<double> v, tau;
        dev_->ortho(r.block, v, tau);
        const int ld = plan_.c_cap[r.block];
        out.resize((size_t)r.rows * r.cols);
        for (int j = 0; j < r.cols; j++)
            for (int i = 0; i < r.rows; i++) out[i + (size_t)j * r.rows] = v[i + (size_t)j * ld];
    }
}

void Tree::op_perm(int idx, std::vector<int>& out) const {
    spand::DeviceScope scope(device_);
    const OpRecord& r = ops_.at(idx);
    out.clear();
    if (r.kind != 8 && r.kind != 9) return;
    if (r.block < 0) {  // sibling: identity
        out.resize(r.ns);
        for (int i = 0; i < r.ns; i++) out[i] = i;
        return;
    }
    dev_->lu_perm(r.cl, out);
    out.resize(r.ns);
}

void Tree::op_signs(int idx, std::vector<double>& out) const {
    spand::DeviceScope scope(device_);
    const OpRecord& r = ops_.at(idx);
    out.clear();
    if (r.kind != 9) return;
    dev_->ldlt_signs(r.cl, out);
    out.resize(r.ns);
}

void Tree::op_tau(int idx, std::vector<double>& out) const {
    spand::DeviceScope scope(device_);
    const OpRecord& r = ops_.at(idx);
    out.clear();
    if (r.kind != 3) return;
    std::vector<double> v, tau;
    dev_->ortho(r.block, v, tau);
    out.assign(tau.begin(), tau.begin() + r.cols);
}

static void add_work(std::vector<Tree::Work>& w, const char* cls, double bytes, double flops) {
    for (auto& e : w)
        if (e.cls == cls) {
            e.bytes += bytes;
            e.flops += flops;
            return;
        }
    w.push_back({cls, bytes, flops});
}

std::vector<Tree::Work> Tree::work_factor() const {
    std::vector<Work> w;
    if (!factored_) return w;
    ensure_log();
    const spand::Plan& P = plan_;
    const double sz = dev_->precision_bytes();
    auto r0 = [&](int c) { return (double)rows0_[c]; };
    for (int l = 0; l < P.nlevels; l++) {
        const spand::LevelPlan& L = P.levels[l];
        auto potrf = [&](const std::vector<int>& cl) {
            for (int c : cl) {
                double n = r0(c);
                add_work(w, "potrf", 2 * n * n * sz, n * n * n / 3);
            }
        };
        auto trsm = [&](const std::vector<spand::TrsmItem>& items) {
            for (const auto& t : items) {
                const spand::PlanBlock& B = P.blocks[t.block];
                double n = r0(t.cluster);
                double m = t.side == 0 ? r0(B.colc) : r0(B.rowc);
                add_work(w, "trsm", (2 * m * n + n * (n + 1) / 2) * sz, m * n * n);
            }
        };
        potrf(L.elim_clusters);
        trsm(L.elim_trsm);
        for (int t = 0; t < L.schur_count; t++) {
            const spand::SchurTarget& st = P.schur_targets[L.schur_first + t];
            const spand::PlanBlock& B = P.blocks[st.target];
            double M = r0(B.rowc), N = r0(B.colc);
            double bytes = 2 * M * N * sz, flops = 0;
            for (int u = 0; u < st.count; u++) {
                double S = r0(P.schur_updates[st.first + u].s);
                bytes += (M + N) * S * sz;
                flops += st.syrk ? M * M * S : 2 * M * N * S;
            }
            add_work(w, "schur", bytes, flops);
        }
        potrf(L.scale_clusters);
        trsm(L.scale_trsm);
        std::map<int, int> wave_of;
        for (size_t wv = 0; wv < L.waves.size(); wv++)
            for (const auto& it : L.waves[wv]) wave_of[it.cluster] = (int)wv;
        for (const auto& wave : L.waves)
            for (const auto& it : wave) {
                double rows = r0(it.cluster), k = csize_[it.cluster], cols = 0;
                for (int p = 0; p < it.count; p++) {
                    int n = P.asn_pieces[it.first + p].nbr;
                    auto wn = wave_of.find(n);
                    cols += (wn != wave_of.end() && wn->second < wave_of[it.cluster]) ? csize_[n] : rows0_[n];
                }
                double kk = std::min(k, std::min(rows, cols));
                add_work(w, "asn_gather", 2 * rows * cols * sz, 0);
                add_work(w, "qrcp", 2 * rows * cols * sz,
                         4 * rows * cols * kk - 2 * kk * kk * (rows + cols) + 4 * kk * kk * kk / 3);
                if (k < rows) add_work(w, "sparsify_scatter", (2 * rows * k + 2 * k * cols) * sz, 0);
            }
        for (const auto& m : L.merge_copies) add_work(w, "merge_copy", 2.0 * csize_[m.nold] * csize_[m.sold] * sz, 0);
    }
    return w;
}

std::vector<Tree::Work> Tree::work_solve() const {
    std::vector<Work> w;
    if (!factored_) return w;
    ensure_log();
    const spand::Plan& P = plan_;
    const double sz = dev_->precision_bytes();
    // both sweeps
    for (int l = 0; l < P.nlevels; l++) {
        const spand::LevelPlan& L = P.levels[l];
        for (int c : L.op_elim_llt) {
            double n = rows0_[c];
            add_work(w, "trsv", 2 * (n * (n + 1) / 2 + 2 * n) * sz, 2 * n * n);
        }
        for (int c : L.op_scale_llt) {
            double n = rows0_[c];
            add_work(w, "trsv", 2 * (n * (n + 1) / 2 + 2 * n) * sz, 2 * n * n);
        }
        for (const auto& g : L.op_gemm) {
            double a = rows0_[g.self], b = rows0_[g.nbr];
            add_work(w, "gemm_fwd", (a * b + a + 2 * b) * sz, 2 * a * b);
            add_work(w, "gemm_bwd", (a * b + 2 * a + b) * sz, 2 * a * b);
        }
        for (int c : L.op_ortho) {
            double rows = rows0_[c], k = csize_[c];
            if (k < rows) add_work(w, "ortho", 2 * (rows * k + 2 * rows) * sz, 2 * 4 * rows * k);
        }
        for (int p : L.op_merge)
            for (int ch : P.c_children[p]) add_work(w, "merge_x", 2 * 2.0 * csize_[ch] * sz, 0);
    }
    const double n = get_N();
    add_work(w, "perm", 2 * n * (8 + 4 + 8 + sz), 0);
    return w;
}

spand::PcgResult Tree::adjoint_device(const double* g, const double* x, double* lambda, double* grad_vals,
                                      int iters, double tol) const {
    spand::DeviceScope scope(device_);
    if (!dev_ || !factored_) throw std::logic_error("adjoint before factorize");
    const size_t nnz = A_.rowval.size();
    if (!d_prow_) {
        std::vector<int> cols(nnz);
        for (int j = 0; j < A_.n; j++)
            for (int k = A_.colptr[j]; k < A_.colptr[j + 1]; k++) cols[k] = j;
        cuda_check(cudaMalloc(&d_prow_, std::max<size_t>(nnz, 1) * sizeof(int)), "cudaMalloc");
        cuda_check(cudaMalloc(&d_pcol_, std::max<size_t>(nnz, 1) * sizeof(int)), "cudaMalloc");
        cuda_check(cudaMemcpy(d_prow_, A_.rowval.data(), nnz * sizeof(int), cudaMemcpyHostToDevice), "H2D");
        cuda_check(cudaMemcpy(d_pcol_, cols.data(), nnz * sizeof(int), cudaMemcpyHostToDevice), "H2D");
    }
    spand::PcgResult r;
    try {
        r = spand::device_pcg(*dev_, dA_, g, lambda, iters, tol, true);
    } catch (spand::DeviceError& e) {
        throw std::runtime_error(e.msg);
    }
    spand::device_pattern_outer(d_prow_, d_pcol_, (int64_t)nnz, lambda, x, grad_vals, stream_);
    dev_->add_launches(1);
    cuda_check(cudaGetLastError(), "adjoint scatter");
    cuda_check(cudaStreamSynchronize(stream_), "sync");
    return r;
}

int cg(const Csc& A, const double* rhs, double* x, const Tree& precond, int iters, double tol, bool verb,
       double* relres) {
    spand::DeviceScope scope(precond.device_id());
    (void)A;  // the tree holds the device copy of the assembled matrix
    const int n = precond.get_N();
    double* db = precond.cg_buffer(0, n);
    double* dx = precond.cg_buffer(1, n);
    cudaStream_t s = precond.stream();
    cuda_check(cudaMemcpyAsync(db, rhs, n * sizeof(double), cudaMemcpyHostToDevice, s), "H2D");
    cuda_check(cudaMemcpyAsync(dx, x, n * sizeof(double), cudaMemcpyHostToDevice, s), "H2D");
    spand::PcgResult r;
    try {
        r = spand::device_pcg(*precond.device(), precond.device_csr(), db, dx, iters, tol, true);
    } catch (spand::DeviceError& e) {
        throw std::runtime_error(e.msg);
    }
    cuda_check(cudaMemcpyAsync(x, dx, n * sizeof(double), cudaMemcpyDeviceToHost, s), "D2H");
    cuda_check(cudaStreamSynchronize(s), "sync");
    if (verb) printf("# of iter:  %d\n", r.iterations);
    if (relres) *relres = r.relres;
    return r.iterations;
}

// GMRES and IR: host vectors through the tree's device buffers
template <typename F>
static spand::PcgResult krylov_host(const Tree& precond, const double* rhs, double* x, F&& run) {
    spand::DeviceScope scope(precond.device_id());
    const int n = precond.get_N();
    double* db = precond.cg_buffer(0, n);
    double* dx = precond.cg_buffer(1, n);
    cudaStream_t s = precond.stream();
    cuda_check(cudaMemcpyAsync(db, rhs, n * sizeof(double), cudaMemcpyHostToDevice, s), "H2D");
    cuda_check(cudaMemcpyAsync(dx, x, n * sizeof(double), cudaMemcpyHostToDevice, s), "H2D");
    spand::PcgResult r;
    try {
        r = run(db, dx);
    } catch (spand::DeviceError& e) {
        throw std::runtime_error(e.msg);
    }
    cuda_check(cudaMemcpyAsync(x, dx, n * sizeof(double), cudaMemcpyDeviceToHost, s), "D2H");
    cuda_check(cudaStreamSynchronize(s), "sync");
    return r;
}

int gmres(const Csc& A, const double* rhs, double* x, const Tree& precond, int iters, int restart, double tol,
          bool verb, double* relres) {
    (void)A;
    if (!precond.device()) throw std::logic_error("gmres before factorize");
    spand::PcgResult r = krylov_host(precond, rhs, x, [&](const double* b, double* xx) {
        return spand::device_gmres(*precond.device(), precond.device_csr(), b, xx, iters, restart, tol);
    });
    if (verb) printf("# of iter:  %d\n", r.iterations);
    if (relres) *relres = r.relres;
    return r.iterations;
}

int fgmres(const Csc& A, const double* rhs, double* x, const Tree& precond, int iters, int restart, double tol,
           bool verb, double* relres) {
    (void)A;
    if (!precond.device()) throw std::logic_error("fgmres before factorize");
    spand::PcgResult r = krylov_host(precond, rhs, x, [&](const double* b, double* xx) {
        return spand::device_fgmres(*precond.device(), precond.device_csr(), b, xx, iters, restart, tol);
    });
    if (verb) printf("# of iter:  %d\n", r.iterations);
    if (relres) *relres = r.relres;
    return r.iterations;
}

int ir(const Csc& A, const double* rhs, double* x, const Tree& precond, int iters, double tol, bool verb,
       double* relres) {
    (void)A;
    if (!precond.device()) throw std::logic_error("ir before factorize");
    spand::PcgResult r = krylov_host(precond, rhs, x, [&](const double* b, double* xx) {
        return spand::device_ir(*precond.device(), precond.device_csr(), b, xx, iters, tol);
    });
    if (verb) printf("# of iter:  %d\n", r.iterations);
    if (relres) *relres = r.relres;
    return r.iterations;
}

void cg_multi(const Tree& precond, const double* rhs, double* x, int nrhs, int ld, int iters, double tol,
              int* iters_out, double* relres_out) {
    spand::DeviceScope scope(precond.device_id());
    const int n = precond.get_N();
    if (nrhs <= 0) return;
    if (ld < n) throw std::invalid_argument("leading dimension smaller than the matrix order");
    const size_t tot = (size_t)n * nrhs;
    double* db = precond.cg_buffer(0, (int)tot);
    double* dx = precond.cg_buffer(1, (int)tot);
    cudaStream_t s = precond.stream();
    const size_t row = (size_t)n * sizeof(double), pitch = (size_t)ld * sizeof(double);
    cuda_check(cudaMemcpy2DAsync(db, row, rhs, pitch, row, nrhs, cudaMemcpyHostToDevice, s), "H2D");
    cuda_check(cudaMemcpy2DAsync(dx, row, x, pitch, row, nrhs, cudaMemcpyHostToDevice, s), "H2D");
    try {
        spand::device_pcg_multi(*precond.device(), precond.device_csr(), db, dx, nrhs, iters, tol, true, iters_out,
                                relres_out);
    } catch (spand::DeviceError& e) {
        throw std::runtime_error(e.msg);
    }
    cuda_check(cudaMemcpy2DAsync(x, pitch, dx, row, row, nrhs, cudaMemcpyDeviceToHost, s), "D2H");
    cuda_check(cudaStreamSynchronize(s), "sync");
}

void batch_factorize(Tree* const* trees, int count, int* status, std::string* messages) {
    std::vector<bool> queued(count, false);
    for (int k = 0; k < count; k++) {
        status[k] = 0;
        try {
            trees[k]->factorize_enqueue();
            queued[k] = true;
        } catch (std::exception& e) {
            status[k] = 1;
            if (messages) messages[k] = e.what();
        }
    }
    for (int k = 0; k < count; k++) {
        if (!queued[k]) continue;
        try {
            trees[k]->factorize_finish();
        } catch (std::exception& e) {
            status[k] = 1;
            if (messages) messages[k] = e.what();
        }
    }
}

// The trees of one batched CG share one device (their lockstep loop runs on it).
static int batch_device(Tree* const* trees, int count) {
    const int dev = count > 0 ? trees[0]->device_id() : -1;
    for (int k = 1; k < count; k++)
        if (trees[k]->device_id() != dev) throw std::invalid_argument("the trees of a batch live on different devices");
    return dev;
}

void batch_cg(Tree* const* trees, int count, const double* const* rhs, double* const* x, int iters, double tol,
              int* iters_out, double* relres_out) {
    spand::DeviceScope scope(batch_device(trees, count));
    std::vector<spand::PcgSystem> sys(count);
    std::vector<double*> db(count), dx(count);
    for (int k = 0; k < count; k++) {
        const Tree& t = *trees[k];
        if (!t.device()) throw std::logic_error("cg before factorize");
        const int n = t.get_N();
        db[k] = t.cg_buffer(0, n);
        dx[k] = t.cg_buffer(1, n);
        cuda_check(cudaMemcpyAsync(db[k], rhs[k], n * sizeof(double), cudaMemcpyHostToDevice, t.stream()), "H2D");
        cuda_check(cudaMemcpyAsync(dx[k], x[k], n * sizeof(double), cudaMemcpyHostToDevice, t.stream()), "H2D");
        sys[k] = spand::PcgSystem{t.device(), &t.device_csr(), &t.pcg_work(), db[k], dx[k], spand::PcgResult{}};
    }
    try {
        spand::device_pcg_batch(sys.data(), count, iters, tol, true);
    } catch (spand::DeviceError& e) {
        throw std::runtime_error(e.msg);
    }
    for (int k = 0; k < count; k++) {
        const Tree& t = *trees[k];
        cuda_check(cudaMemcpyAsync(x[k], dx[k], t.get_N() * sizeof(double), cudaMemcpyDeviceToHost, t.stream()), "D2H");
    }
    for (int k = 0; k < count; k++) {
        cuda_check(cudaStreamSynchronize(trees[k]->stream()), "sync");
        iters_out[k] = sys[k].res.iterations;
        relres_out[k] = sys[k].res.relres;
    }
}

void batch_cg_device(Tree* const* trees, int count, const double* const* b_dev, double* const* x_dev, int iters,
                     double tol, int* iters_out, double* relres_out) {
    spand::DeviceScope scope(batch_device(trees, count));
    std::vector<spand::PcgSystem> sys(count);
    for (int k = 0; k < count; k++) {
        const Tree& t = *trees[k];
        if (!t.device()) throw std::logic_error("cg before factorize");
        sys[k] = spand::PcgSystem{t.device(), &t.device_csr(), &t.pcg_work(), b_dev[k], x_dev[k], spand::PcgResult{}};
    }
    try {
        spand::device_pcg_batch(sys.data(), count, iters, tol, true);
    } catch (spand::DeviceError& e) {
        throw std::runtime_error(e.msg);
    }
    for (int k = 0; k < count; k++) {
        iters_out[k] = sys[k].res.iterations;
        relres_out[k] = sys[k].res.relres;
    }
}

}  // namespace spaND

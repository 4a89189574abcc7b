// Forest: many independent SPD systems in one plan (forest.h).
#include "forest.h"

#include <algorithm>
#include <climits>
#include <stdexcept>

namespace spaND {

static void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

Forest::Forest(Tree* const* trees, int count) {
    if (count <= 0 || !trees) throw std::invalid_argument("a forest needs at least one tree");
    const Tree& t0 = *trees[0];
    for (int k = 0; k < count; k++) {
        const Tree* t = trees[k];
        if (!t || !t->assembled()) throw std::logic_error("forest of trees that are not assembled");
        if (t->get_symm_kind() != SymmKind::SPD) throw std::invalid_argument("a forest holds SPD / LLT systems");
        if (t->get_preserve()) throw std::invalid_argument("a forest does not preserve vectors");
        if (t->is_lorasp()) throw std::invalid_argument("a forest holds spaND trees (partition(), not partition_lorasp())");
        if (t->get_tol() != t0.get_tol() || t->get_skip() != t0.get_skip() || t->get_fp32() != t0.get_fp32() ||
            t->get_use_sparsify() != t0.get_use_sparsify())
            throw std::invalid_argument("the trees of a forest share tolerance, skip, precision and sparsification");
    }
    tol_ = t0.get_tol();
    // stack orderings, hierarchies and matrices; level l of the forest is level l of every tree
    int nl = 0;
    for (int k = 0; k < count; k++) nl = std::max(nl, trees[k]->hierarchy().nlevels);
    H_.nlevels = nl;
    H_.bottoms.resize(nl);
    off_.assign(1, 0);
    nnz_off_.assign(1, 0);
    cluster_off_.assign(1, 0);
    A_.colptr.assign(1, 0);
    for (int k = 0; k < count; k++) {
        const spand::Hierarchy& h = trees[k]->hierarchy();
        const Csc& A = trees[k]->matrix();
        const std::vector<int>& p = trees[k]->get_assembly_perm();
        const int co = cluster_off_.back();
        const long long d = off_.back();
        const int nc = (int)h.start.size();
        for (int c = 0; c < nc; c++) {
            H_.start.push_back(h.start[c] + (int)d);
            H_.size.push_back(h.size[c]);
            H_.level.push_back(h.level[c]);
            H_.sparsify.push_back(h.sparsify[c]);
            H_.parent.push_back(h.parent[c] < 0 ? -1 : h.parent[c] + co);
            H_.hlevel.push_back(h.hlevel[c]);
            std::vector<int> ch(h.children[c]);
            for (int& x : ch) x += co;
            H_.children.push_back(ch);
        }
        for (int l = 0; l < h.nlevels; l++)
            for (int c : h.bottoms[l]) H_.bottoms[l].push_back(c + co);
        for (int i : p) perm_.push_back(i + (int)d);
        for (int j = 0; j < A.n; j++) {
            for (int q = A.colptr[j]; q < A.colptr[j + 1]; q++) {
                A_.rowval.push_back(A.rowval[q] + (int)d);
                A_.val.push_back(A.val[q]);
            }
            A_.colptr.push_back((int)A_.rowval.size());
        }
        if ((long long)A_.rowval.size() > INT32_MAX) throw std::invalid_argument("forest too large");
        off_.push_back(d + A.n);
        nnz_off_.push_back((long long)A_.rowval.size());
        cluster_off_.push_back(co + nc);
    }
    A_.n = (int)off_.back();
    Csc App = spand::symm_perm(A_, perm_);
    asmb_ = spand::assembly_structure(H_, App, true);
    plan_ = spand::build_plan(H_, asmb_, t0.get_skip(), t0.get_use_sparsify(), false);
    std::vector<int64_t> amap = spand::assembly_map(plan_, H_, asmb_, A_, perm_);
    // the forest lives on the device current at its creation
    device_ = spand::current_device();
    check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
    dev_ = spand::make_device_factor(t0.get_fp32(), stream_, perm_);
    try {
        dev_->upload(plan_, amap);
    } catch (spand::DeviceError& e) {
        throw std::runtime_error(e.msg);
    }
    upload_csr(A_, dA_, &d_cmap_);
    std::vector<int> seg(A_.n);
    for (int k = 0; k < count; k++)
        for (long long i = off_[k]; i < off_[k + 1]; i++) seg[i] = k;
    check(cudaMalloc(&d_off_, off_.size() * sizeof(long long)), "cudaMalloc");
    check(cudaMalloc(&d_seg_, std::max<size_t>(seg.size(), 1) * sizeof(int)), "cudaMalloc");
    check(cudaMemcpy(d_off_, off_.data(), off_.size() * sizeof(long long), cudaMemcpyHostToDevice), "H2D");
    check(cudaMemcpy(d_seg_, seg.data(), seg.size() * sizeof(int), cudaMemcpyHostToDevice), "H2D");
    assemble_values(A_.val.data(), (int64_t)A_.val.size(), false);
}

Forest::~Forest() {
    spand::DeviceScope scope(device_);
    dev_.reset();
    work_.release();
    for (auto& p : buf_)
        if (p) cudaFree(p);
    if (d_cmap_) cudaFree(d_cmap_);
    if (d_off_) cudaFree(d_off_);
    if (d_seg_) cudaFree(d_seg_);
    if (dA_.rowptr) cudaFree(dA_.rowptr);
    if (dA_.colind) cudaFree(dA_.colind);
    if (dA_.val) cudaFree(dA_.val);
    if (stream_) cudaStreamDestroy(stream_);
}

void Forest::assemble_values(const double* vals, int64_t nnz, bool on_device) {
    spand::DeviceScope scope(device_);
    if (nnz != (int64_t)A_.rowval.size()) throw std::invalid_argument("values do not match the stacked patterns");
    try {
        dev_->assemble_values(vals, nnz, on_device);
    } catch (spand::DeviceError& e) {
        throw std::runtime_error(e.msg);
    }
    spand::device_scatter(dev_->device_values(), d_cmap_, nnz, dA_.val, stream_);
    check(cudaGetLastError(), "assembly scatter");
    check(cudaStreamSynchronize(stream_), "sync");
    factored_ = false;
}

void Forest::factorize_enqueue() {
    spand::DeviceScope scope(device_);
    try {
        dev_->factorize_enqueue(tol_);
    } catch (spand::DeviceError& e) {
        throw std::runtime_error(e.msg);
    }
}

void Forest::factorize_finish() {
    spand::DeviceScope scope(device_);
    failed_system_ = -1;
    try {
        dev_->factorize_finish();
    } catch (spand::DeviceError& e) {
        const int c = dev_->failed_cluster();
        if (c >= 0)
            failed_system_ = (int)(std::upper_bound(cluster_off_.begin(), cluster_off_.end(), c) - cluster_off_.begin()) - 1;
        if (e.status == spand::SPAND_ERR_NOT_SPD)
            throw std::runtime_error("Error: Non-SPD Pivot (system " + std::to_string(failed_system_) + ")\n");
        throw std::runtime_error(e.msg);
    }
    factored_ = true;
}

void Forest::factorize() {
    factorize_enqueue();
    factorize_finish();
}

void Forest::solve_device(double* x) const {
    spand::DeviceScope scope(device_);
    if (!factored_) throw std::logic_error("solve before factorize");
    try {
        dev_->solve_device(x, 1, N());
    } catch (spand::DeviceError& e) {
        throw std::runtime_error(e.msg);
    }
}

void Forest::cg_device(const double* b, double* x, int iters, double tol, int* iters_out, double* relres_out) {
    spand::DeviceScope scope(device_);
    if (!factored_) throw std::logic_error("cg before factorize");
    try {
        spand::device_pcg_segmented(*dev_, dA_, b, x, count(), d_off_, off_.data(), d_seg_, work_, iters, tol,
                                    iters_out, relres_out);
    } catch (spand::DeviceError& e) {
        throw std::runtime_error(e.msg);
    }
}

void Forest::cg(const double* b, double* x, int iters, double tol, int* iters_out, double* relres_out) {
    spand::DeviceScope scope(device_);
    const size_t n = (size_t)N();
    for (auto& p : buf_)
        if (!p) check(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(double)), "cudaMalloc");
    check(cudaMemcpyAsync(buf_[0], b, n * sizeof(double), cudaMemcpyHostToDevice, stream_), "H2D");
    check(cudaMemcpyAsync(buf_[1], x, n * sizeof(double), cudaMemcpyHostToDevice, stream_), "H2D");
    cg_device(buf_[0], buf_[1], iters, tol, iters_out, relres_out);
    check(cudaMemcpyAsync(x, buf_[1], n * sizeof(double), cudaMemcpyDeviceToHost, stream_), "D2H");
    check(cudaStreamSynchronize(stream_), "sync");
}

std::vector<std::array<int, 5>> Forest::ranks() const {
    spand::DeviceScope scope(device_);
    std::vector<int> cs, r0;
    dev_->sizes(cs, r0);
    std::vector<std::array<int, 5>> out;
    for (int l = 0; l < plan_.nlevels; l++)
        for (int c : plan_.levels[l].op_ortho) {
            const int k = (int)(std::upper_bound(cluster_off_.begin(), cluster_off_.end(), c) - cluster_off_.begin()) - 1;
            out.push_back({k, l, c - cluster_off_[k], r0[c], cs[c]});
        }
    return out;
}

}  // namespace spaND

// Many independent SPD systems factored and solved as one.
//
// No counterpart in the reference, which factors one matrix per Tree.  A Forest takes K
// partitioned and assembled trees and builds ONE plan for their block-diagonal matrix:
// each system keeps its own nested-dissection ordering and cluster hierarchy (copied from
// its tree), laid side by side, so level l of the plan holds level l of every system.
// Since clusters of different systems never share an edge, every system is eliminated,
// scaled, sparsified and merged exactly as it is alone; what changes is that each launch
// of the fixed sequence carries the work items of all systems (one sequence for the
// deepest system instead of K), and one segmented CG serves all right-hand sides.
#pragma once

#include <array>
#include <memory>
#include <string>
#include <vector>

#include "tree.h"

namespace spaND {

class Forest {
   public:
    // trees: SPD / LLT, partitioned and assembled, with one tolerance, skip, precision and
    // sparsification setting; their orderings, hierarchies and matrices are copied.
    Forest(Tree* const* trees, int count);
    ~Forest();

    int count() const { return (int)off_.size() - 1; }
    // system k: rows [off[k], off[k+1]) of the stacked vectors, in its natural ordering
    const std::vector<long long>& offsets() const { return off_; }
    // system k: values [nnz_off[k], nnz_off[k+1]) of the stacked values (its CSC order)
    const std::vector<long long>& value_offsets() const { return nnz_off_; }
    int N() const { return (int)off_.back(); }

    // new values for every system (stacked, each in the CSC order of its tree's pattern),
    // host or device memory
    void assemble_values(const double* vals, int64_t nnz, bool on_device);
    // throws std::runtime_error naming the first system whose pivot failed
    void factorize();
    void factorize_enqueue();
    void factorize_finish();
    int failed_system() const { return failed_system_; }
    // x <- M^{-1} x on stacked device vectors
    void solve_device(double* x) const;
    // cg (is.cpp:39-121) on every system; b, x stacked, device memory (x: initial guess)
    void cg_device(const double* b, double* x, int iters, double tol, int* iters_out, double* relres_out);
    // the same with host vectors
    void cg(const double* b, double* x, int iters, double tol, int* iters_out, double* relres_out);

    spand::DeviceFactorBase* device() const { return dev_.get(); }
    cudaStream_t stream() const { return stream_; }
    int device_id() const { return device_; }
    int64_t launches() const { return dev_ ? dev_->launches() : 0; }
    void reset_launches() { if (dev_) dev_->reset_launches(); }
    const spand::Plan& plan() const { return plan_; }
    // (system, level, cluster order within its tree, rows, rank) of every sparsified cluster
    std::vector<std::array<int, 5>> ranks() const;

   private:
    std::vector<long long> off_, nnz_off_;
    std::vector<int> cluster_off_;  // system k: clusters [cluster_off[k], cluster_off[k+1])
    spand::Hierarchy H_;
    spand::Assembly asmb_;
    spand::Plan plan_;
    Csc A_;
    std::vector<int> perm_;
    std::unique_ptr<spand::DeviceFactorBase> dev_;
    cudaStream_t stream_ = nullptr;
    int device_ = -1;
    spand::DeviceCsr dA_;
    int* d_cmap_ = nullptr;
    long long* d_off_ = nullptr;
    int* d_seg_ = nullptr;
    double* buf_[2] = {nullptr, nullptr};
    spand::SegPcgWork work_;
    double tol_ = 0;
    bool factored_ = false;
    int failed_system_ = -1;
};

}  // namespace spaND

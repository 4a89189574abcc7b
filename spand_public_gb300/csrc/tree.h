// C++ drop-in for spaND::Tree (include/tree.h:25-197) and the CG driver
// (include/is.h:12-14), backed by the GB300 device factorization.
//
// Eigen types of the reference signatures are replaced by plain CSC arrays and raw
// vectors; names, argument meaning and error behaviour (std::runtime_error on a
// non-SPD pivot, tree.cpp:587-590) follow the reference.
#pragma once

#include <array>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "device.h"
#include "host.h"

namespace spaND {

using spand::ClusterID;
using spand::Csc;
using spand::SepID;

enum class ScalingKind { SVD, PLU, PLUQ, EVD, LLT, LDLT };
enum class PartKind { MND, RB };
enum class SymmKind { SPD, SYM, GEN };

// Per-level record, as Log in include/util.h:366-401 (fields used for parity).
struct LevelLog {
    long long dofs_nd = 0, dofs_left_nd = 0, dofs_left_elim = 0, dofs_left_spars = 0;
    long long rank_before_sum = 0, rank_after_sum = 0, rank_after_count = 0, ignored = 0;
    long long nbrs_sum = 0, nbrs_count = 0, fact_nnz = 0;
};

// One recorded operation of the factor, in the reference's op-list order
// (operations.h:32-163): kind 0 ScalingLLT, 1 GemmSymmOut, 2 GemmSymmIn, 3 Orthogonal,
// 4 Merge, 5 Split, 6 GemmOut, 7 GemmIn, 8 ScalingPLUQ (the last three on the GEN / PLU
// path; the matrix of a ScalingPLUQ is its pivot block: L_s below the diagonal, U_s on and
// above it), 9 ScalingLDLT (SYM / LDLT path; L_s in the lower triangle of its block).
struct OpRecord {
    int kind, level, self, nbr, ns, nn, rows, cols;
    int block;    // device block (ScalingLLT / Gemm), or sparsified cluster (Orthogonal), or -1
    int cl = -1;  // device cluster of self (pivot ops: where its permutation and signs live)
};

class Tree {
   public:
    explicit Tree(int nlevels);
    ~Tree();

    void set_verb(bool v) { verb_ = v; }
    void set_Xcoo(const double* X, int dim, int n);
    void set_use_geo(bool g) { geo_ = g; }
    void set_tol(double t) { tol_ = t; }
    void set_skip(int s) { skip_ = s; }
    void set_scaling_kind(ScalingKind k) { scaling_ = k; }
    void set_symm_kind(SymmKind k) { symm_ = k; }
    void set_part_kind(PartKind k) { part_kind_ = k; }
    void set_use_sparsify(bool u) { use_want_sparsify_ = u; }
    // tree.h:136-137: keep the columns of phi in the range of every sparsification
    // (symmetric kinds only).  phi: n x nphi, column-major, natural ordering; copied (the
    // reference borrows the pointer and reads it in factorize()).
    void set_preserve(bool p) { preserve_ = p; }
    void set_phi(const double* phi, int n, int nphi);
    bool get_preserve() const { return preserve_; }
    // No reference counterpart: storage/arithmetic type of the factor (false: FP64).
    void set_fp32(bool f) { fp32_ = f; }

    std::vector<ClusterID> partition(const Csc& A);
    // LoRaSp (tree.h:177, tree.cpp:421-503): geometric recursive bisection; returns the part
    // of every dof (natural ordering).  Then assemble() and factorize_lorasp().
    std::vector<int> partition_lorasp(const Csc& A);
    // tree.h:187, tree.cpp:1553-1608 (SPD / LLT)
    void factorize_lorasp();
    bool is_lorasp() const { return lorasp_; }
    void assemble(const Csc& A);
    // No counterpart in the reference: new values on the pattern of the last assemble()
    // (CSC order, nnz entries), from host or device memory; the plan and device work lists
    // are reused.  Device values leave the host copy of A (matrix()) unchanged.
    void assemble_values(const double* vals, int64_t nnz, bool on_device);
    // assemble() for the pattern of the last assemble() given as raw CSC arrays: new values
    // without building, validating or comparing a second copy of the matrix; returns false
    // (and does nothing) when the pattern differs or nothing was assembled yet
    bool assemble_same_pattern(int n, const int* colptr, const int* rowval, const double* vals);
    void factorize();
    // factorize() in two halves: every launch queued on the tree's stream, then the wait
    // and the status check (what factorize() does in one call)
    void factorize_enqueue();
    void factorize_finish();
    // work vectors of this tree's device CG
    spand::PcgWork& pcg_work() const;
    // x <- M^{-1} x, host vector(s) in natural ordering (tree.cpp:1610-1635)
    void solve(double* x, int nrhs = 1, int ld = -1) const;
    // device vector(s)
    void solve_device(double* x, int nrhs, int ld) const;
    // device vector(s), allocating nothing (fixed scratch shared by all such calls)
    void solve_device_noalloc(double* x, int nrhs, int ld) const;

    int get_N() const { return (int)perm_.size(); }
    const std::vector<int>& get_assembly_perm() const { return perm_; }
    long long nnz() const;
    int get_stop() const;
    int get_nlevels() const { return nlevels_; }
    const std::vector<LevelLog>& log() const { ensure_log(); return log_; }
    // print_log() (include/tree.h:197, src/tree.cpp:1645-1727): per level the dof counts of
    // the ordering, elimination and sparsification, the factor's stored entries, the
    // ranks before and after sparsification and the neighbour counts, then the phase
    // times of the last partition / assemble / factorize; printed to stdout.
    void print_log() const;
    // (level, cluster order, rows, rank) for every sparsified cluster, reference order
    std::vector<std::array<int, 4>> ranks() const;
    const std::vector<OpRecord>& ops() const { ensure_log(); return ops_; }
    void op_matrix(int idx, std::vector<double>& out) const;
    void op_tau(int idx, std::vector<double>& out) const;
    // row permutation p of a ScalingPLUQ / ScalingLDLT op (x_s <- x_s[p] before L_s^{-1})
    void op_perm(int idx, std::vector<int>& out) const;
    // sign(D) of a ScalingLDLT op
    void op_signs(int idx, std::vector<double>& out) const;
    double t_partition = 0, t_assemble = 0, t_factorize = 0;
    int64_t launches() const { return dev_ ? dev_->launches() : 0; }
    void reset_launches() { if (dev_) dev_->reset_launches(); }
    spand::DeviceFactorBase* device() const { return dev_.get(); }
    const Csc& matrix() const { return A_; }
    const spand::Plan& plan() const { return plan_; }
    const spand::Hierarchy& hierarchy() const { return H_; }
    double get_tol() const { return tol_; }
    int get_skip() const { return skip_; }
    bool get_fp32() const { return fp32_; }
    bool get_use_sparsify() const { return use_want_sparsify_; }
    SymmKind get_symm_kind() const { return symm_; }
    bool assembled() const { return assembled_ok_; }
    cudaStream_t stream() const { return stream_; }
    // CUDA device the tree was assembled on (-1 before the first assemble()); every call
    // that touches the tree's memory makes it current and then restores the caller's
    int device_id() const { return device_; }
    const spand::DeviceCsr& device_csr() const { return dA_; }
    size_t device_bytes() const;
    // device vectors of the CG driver (b, x), kept across calls
    double* cg_buffer(int which, int n) const;

    // Algorithmic work per kernel class for one factorization and for one solve with one
    // right-hand side: (class, bytes, flops).  Bytes count each operand read or written
    // once; flops use the standard LAPACK counts (QRCP truncated at the rank).
    struct Work {
        std::string cls;
        double bytes = 0, flops = 0;
    };
    std::vector<Work> work_factor() const;
    std::vector<Work> work_solve() const;

    // No reference counterpart: factorize + device PCG on device vectors, timed with
    // CUDA events on the tree's stream.  out: factor ms, PCG ms, iterations, |r|/|b|.
    // nrhs right-hand sides: b_dev, x_dev n x nrhs (leading dimension n)
    void bench_step(const double* b_dev, double* x_dev, int nrhs, int iters, double tol, double out[4]);

    // No reference counterpart: the adjoint of x = A^{-1} b for a loss L(x).  lambda =
    // A^{-T} g (g = dL/dx) by the preconditioned Krylov solve with this factor (A SPD:
    // A^{-T} = A^{-1}, PCG), then grad_vals[k] = -lambda[row_k] x[col_k] for every stored
    // entry k of A in the CSC order of the assembled pattern (dL/dvalues); dL/db = lambda.
    // Device vectors; lambda holds the initial guess.
    spand::PcgResult adjoint_device(const double* g, const double* x, double* lambda, double* grad_vals, int iters,
                                    double tol) const;

   private:
    void build_ops_and_log();
    void build_ops_and_log_lorasp();
    std::string pivot_error() const;
    void prepare_factorize();  // hands phi to the device (or turns preservation off)
    void ensure_log() const {
        if (log_dirty_) const_cast<Tree*>(this)->build_ops_and_log();
    }

    int nlevels_;
    bool verb_ = true, geo_ = false, use_want_sparsify_ = true, fp32_ = false;
    bool preserve_ = false;
    bool lorasp_ = false, lorasp_run_ = false;
    std::vector<double> phi_;
    int phi_n_ = 0, nphi_ = 0;
    double tol_ = 10.0;  // tree.cpp:94
    int skip_ = 0;
    ScalingKind scaling_ = ScalingKind::LLT;
    SymmKind symm_ = SymmKind::SPD;
    PartKind part_kind_ = PartKind::MND;
    std::vector<double> X_;
    int dim_ = 0;
    std::vector<ClusterID> part_;
    std::vector<int> perm_;
    spand::Hierarchy H_;
    spand::Assembly asmb_;
    spand::Plan plan_;
    Csc A_;

    std::unique_ptr<spand::DeviceFactorBase> dev_;
    cudaStream_t stream_ = nullptr;
    int device_ = -1;
    spand::DeviceCsr dA_;
    mutable double* dx_ = nullptr;
    mutable size_t dx_len_ = 0;
    mutable double* cg_buf_[2] = {nullptr, nullptr};
    mutable size_t cg_len_ = 0;
    mutable std::unique_ptr<spand::PcgWork> pcg_work_;
    int* d_cmap_ = nullptr;  // CSC entry -> CSR position
    mutable int* d_prow_ = nullptr;  // row / column of every CSC entry (adjoint scatter)
    mutable int* d_pcol_ = nullptr;
    bool partitioned_ = false, assembled_ok_ = false, factored_ = false;
    std::vector<LevelLog> log_;
    std::vector<OpRecord> ops_;
    std::vector<int> csize_, rows0_;
    bool log_dirty_ = false;
};

// CSR copy of A on the device (for the SpMV of the Krylov drivers; A structurally
// symmetric) and the CSR position of every CSC entry (*d_cmap), replacing earlier arrays
void upload_csr(const Csc& A, spand::DeviceCsr& dA, int** d_cmap);

// Preconditioned CG (is.cpp:39-121) on the device; b and x are host vectors.
int cg(const Csc& A, const double* rhs, double* x, const Tree& precond, int iters, double tol, bool verb,
       double* relres = nullptr);

// Restarted GMRES (is.cpp:123-300) with the tree as left preconditioner, on the device;
// rhs, x host vectors (x: initial guess).  relres: |w_k| / |M^{-1} r_0|, the quantity the
// reference's stopping test uses.
int gmres(const Csc& A, const double* rhs, double* x, const Tree& precond, int iters, int restart, double tol,
          bool verb, double* relres = nullptr);

// No counterpart in the reference: flexible (right-preconditioned) restarted GMRES whose
// recurrence residual is the true |b - A x|, for factors stored in FP32; stops when
// |b - A x| < tol |b|.
int fgmres(const Csc& A, const double* rhs, double* x, const Tree& precond, int iters, int restart, double tol,
           bool verb, double* relres = nullptr);

// Iterative refinement (is.cpp:12-37) on the device; relres = |b - A x| / |b|.
int ir(const Csc& A, const double* rhs, double* x, const Tree& precond, int iters, double tol, bool verb,
       double* relres = nullptr);

// No counterpart in the reference: cg on nrhs right-hand sides at once (independent CGs
// in lockstep, one multi-right-hand-side preconditioner application per iteration).
// rhs, x: host n x nrhs, leading dimension ld; per column the iteration count and |r|/|b|.
void cg_multi(const Tree& precond, const double* rhs, double* x, int nrhs, int ld, int iters, double tol,
              int* iters_out, double* relres_out);

// No counterpart in the reference: factorize many trees at once (every tree's launches
// queued on its own stream before the first wait); status[k]: 0 or the error of tree k.
void batch_factorize(Tree* const* trees, int count, int* status, std::string* messages);

// No counterpart in the reference: cg on many independent systems at once (tree k with
// rhs[k] -> x[k], host vectors of the tree's size), advanced in lockstep with one host
// wait per iteration for all systems.
void batch_cg(Tree* const* trees, int count, const double* const* rhs, double* const* x, int iters, double tol,
              int* iters_out, double* relres_out);
// batch_cg on device vectors (b_dev[k], x_dev[k]: the tree's size, x holds the initial guess)
void batch_cg_device(Tree* const* trees, int count, const double* const* b_dev, double* const* x_dev, int iters,
                     double tol, int* iters_out, double* relres_out);

}  // namespace spaND

// Device numeric factorization and solve for the GB300 spaND path.
//
// The plan (host.h) fixes every work list; this layer uploads them once and runs the
// factorization as a fixed launch sequence on one stream.  Cluster sizes live in device
// memory: the QRCP kernels shrink them, later kernels read them, so no host round trip
// happens inside factorize().  T is the storage/arithmetic type of the factor (double
// for the plain path, float for the mixed path).
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "host.h"

namespace spand {

// Status codes shared with the C ABI.
enum Status : int {
    SPAND_OK = 0,
    SPAND_ERR_ARG = 1,
    SPAND_ERR_STATE = 2,
    SPAND_ERR_CUDA = 3,
    SPAND_ERR_NOT_SPD = 4,
    SPAND_ERR_UNSUPPORTED = 5,
    SPAND_ERR_NO_CONVERGENCE = 6,
};

struct DeviceError {
    int status;
    std::string msg;
};

// Makes `dev` the current CUDA device for the scope's lifetime and gives the caller its
// own device back afterwards (dev < 0: the current device is left alone).  A tree records
// the device it was assembled on; every call that touches its memory or stream runs under
// one of these, so a caller that switched devices in between still reaches the tree's.
class DeviceScope {
   public:
    explicit DeviceScope(int dev) {
        if (dev < 0) return;
        if (cudaGetDevice(&prev_) != cudaSuccess) throw DeviceError{SPAND_ERR_CUDA, "cudaGetDevice failed"};
        if (prev_ == dev) {
            prev_ = -1;
            return;
        }
        const cudaError_t e = cudaSetDevice(dev);
        if (e != cudaSuccess) {
            prev_ = -1;
            throw DeviceError{SPAND_ERR_CUDA, std::string("cudaSetDevice(tree device): ") + cudaGetErrorString(e)};
        }
    }
    ~DeviceScope() {
        if (prev_ >= 0) cudaSetDevice(prev_);
    }
    DeviceScope(const DeviceScope&) = delete;
    DeviceScope& operator=(const DeviceScope&) = delete;

   private:
    int prev_ = -1;
};

// The current CUDA device (throws DeviceError on failure).
inline int current_device() {
    int d = 0;
    const cudaError_t e = cudaGetDevice(&d);
    if (e != cudaSuccess) throw DeviceError{SPAND_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e)};
    return d;
}

// Per-launch counters: how many kernels ran, for the bench's gpu_launches claim.
struct LaunchCounter {
    int64_t launches = 0;
};

// Per-kernel-class device time, recorded with CUDA events on the launching stream
// around every launch while enabled.
class KernelProfiler {
   public:
    ~KernelProfiler();
    void enable(bool on) { on_ = on; }
    bool enabled() const { return on_; }
    void begin(cudaStream_t s, const char* cls);
    void end(cudaStream_t s);
    // accumulate recorded pairs into per-class totals (synchronises the events)
    void collect();
    void clear();
    struct Entry {
        std::string cls;
        int64_t launches = 0;
        double ms = 0.0;
    };
    const std::vector<Entry>& totals() const { return totals_; }

   private:
    cudaEvent_t take();
    bool on_ = false;
    std::vector<cudaEvent_t> pool_;
    size_t used_ = 0;
    struct Rec {
        std::string cls;
        cudaEvent_t a, b;
    };
    std::vector<Rec> recs_;
    std::string cur_;
    cudaEvent_t cur_a_ = nullptr;
    std::vector<Entry> totals_;
};

class DeviceFactorBase {
   public:
    virtual ~DeviceFactorBase() {}
    // work lists and block storage of a plan; amap: assembly_map of the matrix pattern
    virtual void upload(const Plan& P, const std::vector<int64_t>& amap) = 0;
    // assemble the level-0 blocks from the values of A (host, CSC order of the pattern):
    // one copy to the device and a scatter through the assembly map
    // values of the assembled pattern (CSC order), host or device memory
    virtual void assemble_values(const double* vals, int64_t nnz, bool on_device = false) = 0;
    // device copy of the last uploaded values of A (CSC order)
    virtual const double* device_values() const = 0;
    // every launch of the factorization on this object's stream, the status read queued
    // behind them; factorize_finish waits for it (throws DeviceError on a non-SPD pivot)
    virtual void factorize_enqueue(double tol) = 0;
    virtual void factorize_finish() = 0;
    void factorize(double tol) {
        factorize_enqueue(tol);
        factorize_finish();
    }
    // x: device pointer, natural ordering, n x nrhs (ld), FP64; in-place M^{-1} x
    virtual void solve_device(double* x, int nrhs, int ld) = 0;
    virtual void sizes(std::vector<int>& csize, std::vector<int>& rows0) = 0;
    virtual void block(int b, std::vector<double>& out) = 0;  // host copy (ld layout)
    virtual void ortho(int c, std::vector<double>& v, std::vector<double>& tau) = 0;
    // PLU path: the row permutation of cluster c's pivot (capacity entries; the first
    // csize[c] are meaningful)
    virtual void lu_perm(int c, std::vector<int>& out) = 0;
    // LDLT path: sign(D) of cluster c's pivot (capacity entries)
    virtual void ldlt_signs(int c, std::vector<double>& out) = 0;
    virtual int precision_bytes() const = 0;
    virtual cudaStream_t stream() const = 0;
    virtual size_t device_bytes() const = 0;
    // cluster of the pivot that failed in the last factorization (-1: none)
    int failed_cluster() const { return failed_cluster_; }
    int64_t launches() const { return launches_; }
    void reset_launches() { launches_ = 0; }
    void add_launches(int64_t k) { launches_ += k; }
    KernelProfiler& profiler() { return prof_; }
    // capture the solve on buffer x as a CUDA graph; solve_device(x, ...) then replays it
    virtual void capture_solve(double* x, int nrhs, int ld) = 0;
    // solve_device with the per-cluster solve vectors in a fixed device array instead of
    // memory allocated by this object (no allocation of any kind on this path)
    virtual void solve_device_noalloc(double* x, int nrhs, int ld) = 0;
    // preservation (tree.h:136-137): the columns of phi (n x nphi, column-major, natural
    // ordering, host memory; copied) are kept by every sparsification of the following
    // factorizations; nphi = 0 turns it off
    virtual void set_phi(const double* phi, int n, int nphi) = 0;
    // The QRCP launch of every sparsification wave, in launch order: level, wave, matrices,
    // row capacity of its largest matrix, blocked rows per lane (0: the unblocked kernel),
    // CTAs per cluster, threads per CTA, dynamic shared memory, and the row count from which
    // the trailing update is vectorised (INT_MAX: never); with the configurations the
    // measuring factorization timed and their times (empty where none was measured).
    struct QrcpWave {
        int conf[9];
        std::vector<std::array<int, 5>> cand;  // rpl, cs, threads, smem, vec_rows
        std::vector<double> ms;
    };
    virtual std::vector<QrcpWave> qrcp_waves() const { return {}; }

   protected:
    int failed_cluster_ = -1;
    int64_t launches_ = 0;
    KernelProfiler prof_;
};

// perm: assembly permutation (b = P^T x <=> b[i] = x[perm[i]])
std::unique_ptr<DeviceFactorBase> make_device_factor(bool fp32, cudaStream_t stream, const std::vector<int>& perm);

// FP64 preconditioned CG on the device (src/is.cpp:39-121), A in CSR on the device.
struct DeviceCsr {
    int n = 0;
    int* rowptr = nullptr;
    int* colind = nullptr;
    double* val = nullptr;
};

struct PcgResult {
    int iterations = 0;
    double relres = 0.0;  // recurrence residual |r|/|b|
};

PcgResult device_pcg(DeviceFactorBase& M, const DeviceCsr& A, const double* b, double* x, int maxit, double tol,
                     bool use_graph);

// Work vectors of one device CG (n doubles each, scalars on the device and pinned on the host)
struct PcgWork {
    int n = 0;
    double *r = nullptr, *p = nullptr, *z = nullptr, *tmp = nullptr, *partial = nullptr, *sc = nullptr;
    double* h_sc = nullptr;
    ~PcgWork() { release(); }
    void release();
    void ensure(int n);
};

// One system of a batch: its preconditioner, matrix, work vectors, b and x (device,
// FP64, natural ordering); res receives its iterations and |r|/|b|.
struct PcgSystem {
    DeviceFactorBase* M;
    const DeviceCsr* A;
    PcgWork* w;
    const double* b;
    double* x;
    PcgResult res;
};

// device_pcg on `count` independent systems in lockstep (one host wait per iteration for
// all of them); each system runs on its preconditioner's stream.
void device_pcg_batch(PcgSystem* sys, int count, int maxit, double tol, bool use_graph);

// k independent PCGs in lockstep sharing one multi-right-hand-side preconditioner
// application per iteration; b, x: n x k (column j at offset j * n), device memory.
// Per column: iterations and recurrence residual |r|/|b|.
void device_pcg_multi(DeviceFactorBase& M, const DeviceCsr& A, const double* b, double* x, int k, int maxit,
                      double tol, bool use_graph, int* iters_out, double* relres_out);

void device_spmv(const DeviceCsr& A, const double* x, double* y, cudaStream_t s);

// Work of the segmented PCG: n-vectors and per-system scalars (device and pinned host)
struct SegPcgWork {
    int n = 0, k = 0;
    double *r = nullptr, *p = nullptr, *z = nullptr, *Ap = nullptr, *sc = nullptr, *h_sc = nullptr;
    int *active = nullptr, *h_active = nullptr;
    ~SegPcgWork() { release(); }
    void release();
    void ensure(int n, int k);
};

// cg (is.cpp:39-121) on nseg independent systems stored as consecutive segments of one
// vector (system s: rows [off[s], off[s+1]); seg[i]: the system of row i; device arrays;
// off_host: the same offsets on the host) and preconditioned by M, one factor of their
// block-diagonal matrix A.  Per
// iteration one SpMV, one preconditioner application and per-system dots serve all
// systems; a converged system stops changing.  Per system: iterations and |r|/|b|.
void device_pcg_segmented(DeviceFactorBase& M, const DeviceCsr& A, const double* b, double* x, int nseg,
                          const long long* off, const long long* off_host, const int* seg, SegPcgWork& w, int maxit,
                          double tol, int* iters_out, double* relres_out);

// Restarted GMRES (is.cpp:123-300), left preconditioned by M, on the device; b, x device
// vectors (x: initial guess).  relres: the reference's stopping quantity |w_k| / |M^{-1} r_0|.
PcgResult device_gmres(DeviceFactorBase& M, const DeviceCsr& A, const double* b, double* x, int maxit, int restart,
                       double tol);

// Flexible (right-preconditioned) restarted GMRES, no reference counterpart: the
// recurrence residual is the true |b - A x| whatever the factor's precision, so an FP32
// factor reaches an FP64 tolerance; stops when |b - A x| < tol |b| (relres: that ratio).
PcgResult device_fgmres(DeviceFactorBase& M, const DeviceCsr& A, const double* b, double* x, int maxit, int restart,
                        double tol);

// Iterative refinement (is.cpp:12-37) on the device; relres = |b - A x| / |b|.
PcgResult device_ir(DeviceFactorBase& M, const DeviceCsr& A, const double* b, double* x, int maxit, double tol);

// dst[map[k]] = src[k] for map[k] >= 0 (device arrays), on stream s
void device_scatter(const double* src, const int* map, int64_t n, double* dst, cudaStream_t s);

// out[k] = -lam[rows[k]] * x[cols[k]] for k < nnz (device arrays), on stream s
void device_pattern_outer(const int* rows, const int* cols, int64_t nnz, const double* lam, const double* x,
                          double* out, cudaStream_t s);

}  // namespace spand

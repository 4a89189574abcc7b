// spaND CPU oracle -- TEST INFRASTRUCTURE ONLY.
//
// A plain C++ restatement of the reference hot path (leopoldcambier/spaND_public):
// ordering (geometric modified nested dissection), assembly, the level loop of
// Tree::factorize (eliminate / scale / sparsify / merge), the op-replay solve and the
// CG / IR drivers.  Only the test-suite, smoke() and bench.py's CPU baseline legs may
// load this library; the product path never does.
//
// Dense arithmetic: the reference calls OpenBLAS/MKL (dpotrf, dtrsm, dgemm, dsyrk,
// dgeqp3, dormqr, dtrsv, dgemv, dgetrf).  Those libraries are not part of the
// reference tree, so their published algorithms (LAPACK 3.x dpotf2, dgetf2, dlaqp2 with
// the LAWN 176 partial-norm downdating safeguard, dlarfg/dlarf, reference BLAS loops)
// are restated below.  They agree with LAPACK up to rounding; tests compare them with
// scipy's LAPACK on random inputs.
//
// Structure is mirrored exactly (std::list edge lists, insertion and sort orders), since
// edge order decides the column order of the sparsification matrix and therefore the
// QRCP pivot sequence.
//
// Citations are path:line into the reference project.

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <dlfcn.h>
#include <functional>
#include <limits>
#include <list>
#include <map>
#include <memory>
#include <numeric>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

namespace orc {

// ---------------------------------------------------------------------------------
// Dense column-major matrix
// ---------------------------------------------------------------------------------
struct Mat {
    int r = 0, c = 0;
    std::vector<double> v;
    Mat() {}
    Mat(int r_, int c_) : r(r_), c(c_), v((size_t)r_ * (size_t)c_, 0.0) {}
    double& operator()(int i, int j) { return v[(size_t)i + (size_t)j * r]; }
    double operator()(int i, int j) const { return v[(size_t)i + (size_t)j * r]; }
    double* col(int j) { return v.data() + (size_t)j * r; }
    const double* col(int j) const { return v.data() + (size_t)j * r; }
    static Mat eye(int n) {
        Mat I(n, n);
        for (int i = 0; i < n; i++) I(i, i) = 1.0;
        return I;
    }
};
using pMat = std::unique_ptr<Mat>;

static double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// ---------------------------------------------------------------------------------
// Restated dense kernels (util.cpp:122-452 call sites)
// ---------------------------------------------------------------------------------

// Euclidean norm, scaled sum of squares (reference BLAS dnrm2).
static double nrm2(int n, const double* x) {
    if (n < 1) return 0.0;
    if (n == 1) return std::fabs(x[0]);
    double scale = 0.0, ssq = 1.0;
    for (int i = 0; i < n; i++) {
        if (x[i] != 0.0) {
            double a = std::fabs(x[i]);
            if (scale < a) {
                ssq = 1.0 + ssq * (scale / a) * (scale / a);
                scale = a;
            } else {
                ssq += (a / scale) * (a / scale);
            }
        }
    }
    return scale * std::sqrt(ssq);
}

// ---------------------------------------------------------------------------------
// Optional BLAS / LAPACK (timing only).  The reference calls cblas / LAPACKE for its dense
// kernels (util.cpp:122-394).  For the timed CPU baseline the oracle can do the same through
// a CBLAS / LAPACKE library loaded at run time (orc_use_lapack); the parity checks keep the
// restated kernels below, whose QRCP pivots follow the deterministic tie rule.
// ---------------------------------------------------------------------------------
namespace lapk {
using gemm_t = void (*)(int, int, int, int, int, int, double, const double*, int, const double*, int, double,
                        double*, int);
using syrk_t = void (*)(int, int, int, int, int, double, const double*, int, double, double*, int);
using trsm_t = void (*)(int, int, int, int, int, int, int, double, const double*, int, double*, int);
using potrf_t = int (*)(int, char, int, double*, int);
using geqp3_t = int (*)(int, int, int, double*, int, int*, double*);
using threads_t = void (*)(int);
static gemm_t gemm = nullptr;
static syrk_t syrk = nullptr;
static trsm_t trsm = nullptr;
static potrf_t potrf = nullptr;
static geqp3_t geqp3 = nullptr;
// CBLAS / LAPACKE enumerators (public cblas.h / lapacke.h)
enum { ColMajor = 102, NoTrans = 111, Trans = 112, Upper = 121, Lower = 122, NonUnit = 131, Left = 141, Right = 142 };
}  // namespace lapk

// Lower Cholesky, A = L L^T in place (dpotrf 'L'); util.cpp:158-165.  Returns LAPACK info.
static int potf(Mat& A) {
    int n = A.r;
    if (lapk::potrf) return n ? lapk::potrf(lapk::ColMajor, 'L', n, A.v.data(), n) : 0;
    for (int j = 0; j < n; j++) {
        double ajj = A(j, j);
        if (!(ajj > 0.0) || std::isnan(ajj)) return j + 1;
        ajj = std::sqrt(ajj);
        A(j, j) = ajj;
        double* cj = A.col(j);
        for (int i = j + 1; i < n; i++) cj[i] /= ajj;
        for (int k = j + 1; k < n; k++) {
            double f = cj[k];
            if (f == 0.0) continue;
            double* ck = A.col(k);
            for (int i = k; i < n; i++) ck[i] -= cj[i] * f;
        }
    }
    return 0;
}

// B <- L^{-1} B, L lower non-unit (dtrsm Left Lower NoTrans); util.cpp:266-274.
static void trsm_left_lower(const Mat& L, Mat& B) {
    int m = B.r, n = B.c;
    if (lapk::trsm) {
        if (m && n)
            lapk::trsm(lapk::ColMajor, lapk::Left, lapk::Lower, lapk::NoTrans, lapk::NonUnit, m, n, 1.0, L.v.data(), L.r,
                       B.v.data(), m);
        return;
    }
    for (int j = 0; j < n; j++) {
        double* b = B.col(j);
        for (int k = 0; k < m; k++) {
            if (b[k] == 0.0) continue;
            b[k] /= L(k, k);
            const double* lk = L.col(k);
            double bk = b[k];
            for (int i = k + 1; i < m; i++) b[i] -= bk * lk[i];
        }
    }
}

// B <- B L^{-T}, L lower non-unit (dtrsm Right Lower Trans); util.cpp:256-264.
static void trsm_right_lower_trans(const Mat& L, Mat& B) {
    int m = B.r, n = B.c;
    if (lapk::trsm) {
        if (m && n)
            lapk::trsm(lapk::ColMajor, lapk::Right, lapk::Lower, lapk::Trans, lapk::NonUnit, m, n, 1.0, L.v.data(), L.r,
                       B.v.data(), m);
        return;
    }
    for (int j = 0; j < n; j++) {
        double* bj = B.col(j);
        double d = 1.0 / L(j, j);
        for (int i = 0; i < m; i++) bj[i] *= d;
        for (int k = j + 1; k < n; k++) {
            double f = L(k, j);
            if (f == 0.0) continue;
            double* bk = B.col(k);
            for (int i = 0; i < m; i++) bk[i] -= bj[i] * f;
        }
    }
}

// B <- B U^{-1}, U upper non-unit (dtrsm Right Upper NoTrans).
static void trsm_right_upper(const Mat& U, Mat& B) {
    int m = B.r, n = B.c;
    if (lapk::trsm) {
        if (m && n)
            lapk::trsm(lapk::ColMajor, lapk::Right, lapk::Upper, lapk::NoTrans, lapk::NonUnit, m, n, 1.0, U.v.data(), U.r,
                       B.v.data(), m);
        return;
    }
    for (int j = 0; j < n; j++) {
        double* bj = B.col(j);
        for (int k = 0; k < j; k++) {
            double f = U(k, j);
            if (f == 0.0) continue;
            const double* bk = B.col(k);
            for (int i = 0; i < m; i++) bj[i] -= f * bk[i];
        }
        double d = 1.0 / U(j, j);
        for (int i = 0; i < m; i++) bj[i] *= d;
    }
}

// C <- C - op(A) op(B)  (dgemm alpha=-1, beta=1); util.cpp:122-138.
static void gemm_sub(const Mat& A, bool tA, const Mat& B, bool tB, Mat& C) {
    int m = C.r, n = C.c;
    int k = tA ? A.r : A.c;
    if (m == 0 || n == 0 || k == 0) return;
    if (lapk::gemm) {
        lapk::gemm(lapk::ColMajor, tA ? lapk::Trans : lapk::NoTrans, tB ? lapk::Trans : lapk::NoTrans, m, n, k, -1.0,
                   A.v.data(), A.r, B.v.data(), B.r, 1.0, C.v.data(), m);
        return;
    }
    for (int j = 0; j < n; j++) {
        double* cj = C.col(j);
        if (!tA) {
            for (int l = 0; l < k; l++) {
                double b = tB ? B(j, l) : B(l, j);
                if (b == 0.0) continue;
                const double* al = A.col(l);
                for (int i = 0; i < m; i++) cj[i] -= al[i] * b;
            }
        } else {
            for (int i = 0; i < m; i++) {
                const double* ai = A.col(i);
                double s = 0.0;
                if (!tB) {
                    const double* bj = B.col(j);
                    for (int l = 0; l < k; l++) s += ai[l] * bj[l];
                } else {
                    for (int l = 0; l < k; l++) s += ai[l] * B(j, l);
                }
                cj[i] -= s;
            }
        }
    }
}

// lower(C) <- lower(C) - op(A) op(A)^T (dsyrk Lower, alpha=-1, beta=1); util.cpp:148-156.
static void syrk_sub_lower(const Mat& A, bool tA, Mat& C) {
    int n = C.r;
    int k = tA ? A.r : A.c;
    if (n == 0 || k == 0) return;
    if (lapk::syrk) {
        lapk::syrk(lapk::ColMajor, lapk::Lower, tA ? lapk::Trans : lapk::NoTrans, n, k, -1.0, A.v.data(), A.r, 1.0,
                   C.v.data(), n);
        return;
    }
    for (int j = 0; j < n; j++) {
        double* cj = C.col(j);
        if (!tA) {
            for (int l = 0; l < k; l++) {
                double b = A(j, l);
                if (b == 0.0) continue;
                const double* al = A.col(l);
                for (int i = j; i < n; i++) cj[i] -= al[i] * b;
            }
        } else {
            const double* aj = A.col(j);
            for (int i = j; i < n; i++) {
                const double* ai = A.col(i);
                double s = 0.0;
                for (int l = 0; l < k; l++) s += ai[l] * aj[l];
                cj[i] -= s;
            }
        }
    }
}

// x <- L^{-1} x or L^{-T} x (dtrsv Lower NonUnit); util.cpp:276-283.
static void trsv_lower(const Mat& L, double* x, int n, bool trans) {
    if (!trans) {
        for (int k = 0; k < n; k++) {
            x[k] /= L(k, k);
            double xk = x[k];
            const double* lk = L.col(k);
            for (int i = k + 1; i < n; i++) x[i] -= xk * lk[i];
        }
    } else {
        for (int k = n - 1; k >= 0; k--) {
            const double* lk = L.col(k);
            double s = x[k];
            for (int i = k + 1; i < n; i++) s -= lk[i] * x[i];
            x[k] = s / L(k, k);
        }
    }
}

// x <- U^{-1} x, U upper non-unit (dtrsv Upper NoTrans NonUnit).
static void trsv_upper(const Mat& U, double* x, int n) {
    for (int k = n - 1; k >= 0; k--) {
        x[k] /= U(k, k);
        double xk = x[k];
        const double* uk = U.col(k);
        for (int i = 0; i < k; i++) x[i] -= xk * uk[i];
    }
}

// x2 <- x2 - A x1 (gemv_notrans, util.cpp:306-315) ; x2 <- x2 - A^T x1 (gemv_trans, util.cpp:317-326)
static void gemv_sub(const Mat& A, bool trans, const double* x1, double* x2) {
    int m = A.r, n = A.c;
    if (m == 0 || n == 0) return;
    if (!trans) {
        for (int j = 0; j < n; j++) {
            double xj = x1[j];
            const double* aj = A.col(j);
            for (int i = 0; i < m; i++) x2[i] -= aj[i] * xj;
        }
    } else {
        for (int j = 0; j < n; j++) {
            const double* aj = A.col(j);
            double s = 0.0;
            for (int i = 0; i < m; i++) s += aj[i] * x1[i];
            x2[j] -= s;
        }
    }
}

// Householder reflector generation (LAPACK dlarfg).  alpha is updated to beta.
static void larfg(int n, double& alpha, double* x, double& tau) {
    if (n <= 1) { tau = 0.0; return; }
    double xnorm = nrm2(n - 1, x);
    if (xnorm == 0.0) { tau = 0.0; return; }
    // beta = -sign(alpha) |(alpha, x)|, with sign(-0) = +1: a zero leading entry is a zero
    // whatever the sign bit that rounding left on it (LAPACK's SIGN would follow the bit)
    double beta = alpha >= 0.0 ? -std::hypot(alpha, xnorm) : std::hypot(alpha, xnorm);
    const double safmin = std::numeric_limits<double>::min() / std::numeric_limits<double>::epsilon();
    int knt = 0;
    if (std::fabs(beta) < safmin) {
        double rsafmn = 1.0 / safmin;
        do {
            knt++;
            for (int i = 0; i < n - 1; i++) x[i] *= rsafmn;
            beta *= rsafmn;
            alpha *= rsafmn;
        } while (std::fabs(beta) < safmin && knt < 20);
        xnorm = nrm2(n - 1, x);
        beta = alpha >= 0.0 ? -std::hypot(alpha, xnorm) : std::hypot(alpha, xnorm);
    }
    tau = (beta - alpha) / beta;
    double scal = 1.0 / (alpha - beta);
    for (int i = 0; i < n - 1; i++) x[i] *= scal;
    for (int j = 0; j < knt; j++) beta *= safmin;
    alpha = beta;
}

// Relative window inside which two partial column norms count as tied (see geqp3).
static const double QRCP_TIE = 1e-7;

// QR with column pivoting, A P = Q R (dgeqp3 -> dlaqp2); util.cpp:383-394.
// jpvt is 0-based on output (util.cpp:392-393 decrements LAPACK's 1-based pivots).
static void geqp3(Mat& A, std::vector<int>& jpvt, std::vector<double>& tau) {
    int m = A.r, n = A.c;
    jpvt.resize(n);
    tau.assign(std::min(m, n), 0.0);
    if (m == 0 || n == 0) return;
    if (lapk::geqp3) {  // LAPACK's own pivot choice (no tie rule): timing only
        std::fill(jpvt.begin(), jpvt.end(), 0);
        lapk::geqp3(lapk::ColMajor, m, n, A.v.data(), m, jpvt.data(), tau.data());
        for (int& j : jpvt) j -= 1;
        return;
    }
    for (int j = 0; j < n; j++) jpvt[j] = j;
    std::vector<double> vn1(n), vn2(n), work(n);
    for (int j = 0; j < n; j++) { vn1[j] = nrm2(m, A.col(j)); vn2[j] = vn1[j]; }
    const double tol3z = std::sqrt(std::numeric_limits<double>::epsilon());
    int mn = std::min(m, n);
    for (int i = 0; i < mn; i++) {
        // pivot: first column whose partial norm is within QRCP_TIE of the largest.
        // Plain idamax (first exact maximum) lets rounding noise decide between columns
        // whose norms are equal in exact arithmetic (mirror-symmetric stencil columns),
        // so any two implementations could pivot differently; the relative tie window
        // makes the choice reproducible across summation orders.
        double best = 0.0;
        for (int j = i; j < n; j++) best = std::max(best, std::fabs(vn1[j]));
        int pvt = i;
        for (int j = i; j < n; j++)
            if (std::fabs(vn1[j]) >= best * (1.0 - QRCP_TIE)) { pvt = j; break; }
        if (pvt != i) {
            std::swap_ranges(A.col(pvt), A.col(pvt) + m, A.col(i));
            std::swap(jpvt[pvt], jpvt[i]);
            vn1[pvt] = vn1[i];
            vn2[pvt] = vn2[i];
        }
        double* ci = A.col(i);
        if (i < m - 1) larfg(m - i, ci[i], ci + i + 1, tau[i]);
        else larfg(1, ci[m - 1], ci + m - 1, tau[i]);
        if (i < n - 1 && tau[i] != 0.0) {
            // apply H(i)^T = H(i) to A(i:m, i+1:n) from the left (dlarf)
            double aii = ci[i];
            ci[i] = 1.0;
            for (int j = i + 1; j < n; j++) {
                double* cj = A.col(j);
                double s = 0.0;
                for (int r = i; r < m; r++) s += ci[r] * cj[r];
                s *= tau[i];
                for (int r = i; r < m; r++) cj[r] -= s * ci[r];
            }
            ci[i] = aii;
        }
        // partial column norm downdating (LAWN 176 safeguard)
        for (int j = i + 1; j < n; j++) {
            if (vn1[j] != 0.0) {
                double temp = std::fabs(A(i, j)) / vn1[j];
                temp = 1.0 - temp * temp;
                temp = std::max(temp, 0.0);
                double r = vn1[j] / vn2[j];
                double temp2 = temp * r * r;
                if (temp2 <= tol3z) {
                    if (i < m - 1) {
                        vn1[j] = nrm2(m - i - 1, A.col(j) + i + 1);
                        vn2[j] = vn1[j];
                    } else {
                        vn1[j] = 0.0;
                        vn2[j] = 0.0;
                    }
                } else {
                    vn1[j] *= std::sqrt(temp);
                }
            }
        }
    }
}

// Apply Q (trans=false) or Q^T (trans=true) of k reflectors stored in v (m x >=k) to x
// (dormqr Left, nrhs=1); util.cpp:328-351.
static void ormqr_vec(const Mat& v, const std::vector<double>& h, int k, double* x, bool trans) {
    int m = v.r;
    if (m == 0 || k == 0) return;
    auto apply = [&](int i) {
        if (h[i] == 0.0) return;
        const double* vi = v.col(i);
        double s = x[i];
        for (int r = i + 1; r < m; r++) s += vi[r] * x[r];
        s *= h[i];
        x[i] -= s;
        for (int r = i + 1; r < m; r++) x[r] -= s * vi[r];
    };
    if (trans) for (int i = 0; i < k; i++) apply(i);
    else for (int i = k - 1; i >= 0; i--) apply(i);
}

// Relative size below which the part of a column left by the previous reflectors counts
// as zero in geqrf (see there).
static const double QR_DEAD = 1e-10;

// Householder QR without pivoting (dgeqrf -> dgeqr2), reflectors below the diagonal,
// tau of size min(m, n); util.cpp:424-432.  Deviation: a column whose remaining part
// A(i:m, i) is below QR_DEAD of its norm (a column that depends on the previous ones, as
// the mirror-image columns of [A_sn phi, phi] on symmetric grids do) gets tau = 0 and is
// left as it is -- dgeqrf would build its reflector from rounding noise, which no two
// summation orders reproduce; the reflectors of the other columns are unchanged.
static void geqrf(Mat& A, std::vector<double>& tau) {
    const int m = A.r, n = A.c, k = std::min(m, n);
    tau.assign(k, 0.0);
    for (int i = 0; i < k; i++) {
        double* ci = A.col(i);
        if (nrm2(m - i, ci + i) <= QR_DEAD * nrm2(m, ci)) continue;
        if (i < m - 1) larfg(m - i, ci[i], ci + i + 1, tau[i]);
        else larfg(1, ci[m - 1], ci + m - 1, tau[i]);
        if (i < n - 1 && tau[i] != 0.0) {
            const double aii = ci[i];
            ci[i] = 1.0;
            for (int j = i + 1; j < n; j++) {
                double* cj = A.col(j);
                double s = 0.0;
                for (int r = i; r < m; r++) s += ci[r] * cj[r];
                s *= tau[i];
                for (int r = i; r < m; r++) cj[r] -= s * ci[r];
            }
            ci[i] = aii;
        }
    }
}

// The first k columns of Q = H_0 ... H_{k-1}, in place over the k reflectors of an m x k
// matrix (dorgqr -> dorg2r order: reflectors applied last to first); util.cpp:372-380.
static void orgqr(Mat& A, const std::vector<double>& tau) {
    const int m = A.r, k = A.c;
    for (int i = k - 1; i >= 0; i--) {
        double* ci = A.col(i);
        if (i < k - 1) {
            ci[i] = 1.0;
            if (tau[i] != 0.0)
                for (int j = i + 1; j < k; j++) {
                    double* cj = A.col(j);
                    double s = 0.0;
                    for (int r = i; r < m; r++) s += ci[r] * cj[r];
                    s *= tau[i];
                    for (int r = i; r < m; r++) cj[r] -= s * ci[r];
                }
        }
        for (int r = i + 1; r < m; r++) ci[r] *= -tau[i];
        ci[i] = 1.0 - tau[i];
        for (int r = 0; r < i; r++) ci[r] = 0.0;
    }
}

// B <- L^T B, L lower triangular (cblas_dtrmm Left Lower Trans NonUnit, rows ascending);
// util.cpp:296-304.
static void trmm_trans(const Mat& L, Mat& B) {
    const int m = B.r;
    for (int j = 0; j < B.c; j++) {
        double* b = B.col(j);
        for (int i = 0; i < m; i++) {
            double t = b[i] * L(i, i);
            for (int k = i + 1; k < m; k++) t += L(k, i) * b[k];
            b[i] = t;
        }
    }
}

// Partial-pivot LU (dgetrf -> dgetf2); returns info; swap is 0-based; util.cpp:183-200.
static int getf(Mat& A, std::vector<int>& perm) {
    int n = A.r;
    std::vector<int> swp(n);
    int info = 0;
    for (int j = 0; j < n; j++) {
        int p = j;
        double best = std::fabs(A(j, j));
        for (int i = j + 1; i < n; i++)
            if (std::fabs(A(i, j)) > best) { best = std::fabs(A(i, j)); p = i; }
        swp[j] = p;
        if (A(p, j) != 0.0) {
            if (p != j)
                for (int c = 0; c < n; c++) std::swap(A(j, c), A(p, c));
            double d = 1.0 / A(j, j);
            for (int i = j + 1; i < n; i++) A(i, j) *= d;
        } else if (info == 0) {
            info = j + 1;
        }
        for (int c = j + 1; c < n; c++) {
            double f = A(j, c);
            if (f == 0.0) continue;
            for (int i = j + 1; i < n; i++) A(i, c) -= A(i, j) * f;
        }
    }
    if (info != 0) return info;
    // swap2perm (util.cpp:76-88)
    perm.resize(n);
    for (int i = 0; i < n; i++) perm[i] = i;
    for (int i = 0; i < n; i++) std::swap(perm[swp[i]], perm[i]);
    return 0;
}

// Eigen's LDLT<MatrixXd, Lower> (Eigen/src/Cholesky/LDLT.h, ldlt_inplace<Lower>::unblocked,
// Eigen 3.3): left-looking LDL^T with symmetric pivoting.  At step k the pivot is the first
// entry of largest magnitude among the diagonal entries k..n-1 as they stand (for j > k not
// yet updated by the earlier columns); the swap touches the lower triangle only.  On exit
// the strict lower triangle holds the unit L, the diagonal holds D, transp[k] the row
// swapped with k.  Returns false where Eigen reports failure: an all-zero diagonal at step
// 0, or a nonzero pivot after a zero one.
// Deviation, as for the QRCP pivots: the pivot is the FIRST entry within a relative
// LDLT_TIE of the largest magnitude.  The sign pivots of the sparsified clusters are +-I
// in exact arithmetic, so after Q^T D Q their diagonals tie up to rounding, and the
// summation order alone would decide Eigen's strict maximum.
static const double LDLT_TIE = 1e-7;
static bool ldlt_eigen(Mat& A, std::vector<int>& transp) {
    const int n = A.r;
    transp.assign(n, 0);
    std::vector<double> temp(n);
    bool ok = true, found_zero = false;
    for (int k = 0; k < n; k++) {
        double bv = 0;
        for (int j = k; j < n; j++) bv = std::max(bv, std::fabs(A(j, j)));
        int big = k;
        for (int j = k; j < n; j++)
            if (std::fabs(A(j, j)) >= bv * (1.0 - LDLT_TIE)) { big = j; break; }
        transp[k] = big;
        if (big != k) {
            for (int c = 0; c < k; c++) std::swap(A(k, c), A(big, c));
            for (int r = big + 1; r < n; r++) std::swap(A(r, k), A(r, big));
            std::swap(A(k, k), A(big, big));
            for (int i = k + 1; i < big; i++) std::swap(A(i, k), A(big, i));
        }
        const int rs = n - k - 1;
        if (k > 0) {
            for (int j = 0; j < k; j++) temp[j] = A(j, j) * A(k, j);
            double d = 0;
            for (int j = 0; j < k; j++) d += A(k, j) * temp[j];
            A(k, k) -= d;
            for (int j = 0; j < k; j++)
                for (int r = k + 1; r < n; r++) A(r, k) -= A(r, j) * temp[j];
        }
        const double akk = A(k, k);
        const bool valid = std::fabs(akk) > 0.0;
        if (k == 0 && !valid) {
            for (int j = 0; j < n; j++) transp[j] = j;
            return false;
        }
        if (rs > 0 && valid) {
            for (int r = k + 1; r < n; r++) A(r, k) /= akk;
        } else if (rs > 0) {
            for (int r = k + 1; r < n; r++) ok = ok && A(r, k) == 0.0;
        }
        if (found_zero && valid) ok = false;
        else if (!valid) found_zero = true;
    }
    return ok;
}

// util.cpp:167-184: L |D|^1/2 (lower, non-unit), sign(D), and the row permutation
// (swap2perm of Eigen's transpositions); returns 1 when Eigen reports failure.
static int ldlt(const Mat& Ass, Mat& L, std::vector<double>& s, std::vector<int>& perm) {
    const int n = Ass.r;
    if (n == 0) return 0;
    Mat A = Ass;
    std::vector<int> tr;
    if (!ldlt_eigen(A, tr)) return 1;
    L = Mat(n, n);
    s.assign(n, 0.0);
    for (int j = 0; j < n; j++) {
        const double dj = A(j, j);
        const double h = std::sqrt(std::fabs(dj));
        s[j] = (dj > 0) - (dj < 0);
        L(j, j) = h;
        for (int i = j + 1; i < n; i++) L(i, j) = A(i, j) * h;
    }
    perm.resize(n);
    for (int i = 0; i < n; i++) perm[i] = i;
    for (int i = 0; i < n; i++) std::swap(perm[tr[i]], perm[i]);
    return 0;
}

// A = L (D + U') -> L |D|^1/2 and |D|^1/2 sign(D) (I + D^-1 U'); util.cpp:212-227.
static void split_LU(const Mat& A, Mat& L, Mat& U) {
    int n = A.r;
    L = Mat(n, n);
    U = Mat(n, n);
    for (int j = 0; j < n; j++) {
        double dj = A(j, j);
        double sj = std::sqrt(std::fabs(dj));
        for (int i = j + 1; i < n; i++) L(i, j) = A(i, j) * sj;
        L(j, j) = sj;
    }
    for (int j = 0; j < n; j++) {
        for (int i = 0; i < j; i++) {
            double di = A(i, i);
            double sgn = (di > 0) - (di < 0);
            U(i, j) = sgn * std::sqrt(std::fabs(di)) * (A(i, j) / di);
        }
        double dj = A(j, j);
        double sgn = (dj > 0) - (dj < 0);
        U(j, j) = sgn * std::sqrt(std::fabs(dj));
    }
}

// Rank from |R_ii| / |R_00| >= tol (prefix); util.cpp:434-452.
static int choose_rank(const std::vector<double>& s, double tol) {
    int n = (int)s.size();
    if (tol == 0) return n;
    if (tol >= 1.0) return 0;
    if (n <= 1) return n;
    double sref = std::fabs(s[0]);
    int rank = 1;
    while (rank < n && std::fabs(s[rank]) / sref >= tol) rank++;
    return rank;
}

// ---------------------------------------------------------------------------------
// Sparse matrix (CSC, sorted rows, no duplicates)
// ---------------------------------------------------------------------------------
struct CSC {
    int n = 0;
    std::vector<int> colptr, rowval;
    std::vector<double> val;
};

// A[p,p]: App(i,j) = A(p[i], p[j]); util.cpp:519-546.
static CSC symm_perm(const CSC& A, const std::vector<int>& p) {
    int n = A.n;
    std::vector<int> pinv(n);
    for (int i = 0; i < n; i++) pinv[p[i]] = i;
    std::vector<int> cnt(n + 1, 0);
    for (int j = 0; j < n; j++) cnt[pinv[j] + 1] += A.colptr[j + 1] - A.colptr[j];
    CSC B;
    B.n = n;
    B.colptr.assign(n + 1, 0);
    for (int j = 0; j < n; j++) B.colptr[j + 1] = B.colptr[j] + cnt[j + 1];
    B.rowval.resize(A.rowval.size());
    B.val.resize(A.val.size());
    std::vector<std::pair<int, double>> tmp;
    for (int jn = 0; jn < n; jn++) {
        int j = p[jn];
        tmp.clear();
        for (int k = A.colptr[j]; k < A.colptr[j + 1]; k++) tmp.push_back({pinv[A.rowval[k]], A.val[k]});
        std::sort(tmp.begin(), tmp.end(), [](auto& a, auto& b) { return a.first < b.first; });
        int o = B.colptr[jn];
        for (size_t t = 0; t < tmp.size(); t++) { B.rowval[o + t] = tmp[t].first; B.val[o + t] = tmp[t].second; }
    }
    return B;
}

// ---------------------------------------------------------------------------------
// Partitioning (partition.h:23-75, partition.cpp)
// ---------------------------------------------------------------------------------
struct SepID {
    int lvl = -1, sep = 0;
    SepID() {}
    SepID(int l, int s) : lvl(l), sep(s) {}
    bool operator==(const SepID& o) const { return lvl == o.lvl && sep == o.sep; }
    bool operator<(const SepID& o) const { return lvl < o.lvl || (lvl == o.lvl && sep < o.sep); }
};
struct ClusterID {
    SepID self, l, r;
    ClusterID() {}
    ClusterID(SepID s, SepID a, SepID b) : self(s), l(a), r(b) {}
    bool operator==(const ClusterID& o) const { return self == o.self && l == o.l && r == o.r; }
    bool operator<(const ClusterID& o) const {
        return (self < o.self) || (self == o.self && l < o.l) || (self == o.self && l == o.l && r < o.r);
    }
};
// partition.cpp:8-16
static SepID merge_sep(const SepID& s) { return SepID(s.lvl + 1, s.sep / 2); }
static ClusterID merge_if(const ClusterID& c, int lvl) {
    SepID left = c.l.lvl < lvl ? merge_sep(c.l) : c.l;
    SepID right = c.r.lvl < lvl ? merge_sep(c.r) : c.r;
    return ClusterID(c.self, left, right);
}

// Geometric ND bisection with one-sided vertex separator; partition.cpp:139-210.
// X is dim x N column-major (X[d + dim*i]).
static void partition_nd_geo(const std::vector<int>& colptr, const std::vector<int>& rowval, const std::vector<int>& dofs,
                             std::vector<int>& parts, const double* X, int dim, std::vector<int>& invp) {
    int N = (int)dofs.size();
    if (N == 0) return;
    int bestdim = -1;
    double maxrange = -1.0;
    for (int d = 0; d < dim; d++) {
        double maxi = std::numeric_limits<double>::lowest();
        double mini = std::numeric_limits<double>::max();
        for (int i = 0; i < N; i++) {
            double x = X[d + (size_t)dim * dofs[i]];
            maxi = std::max(maxi, x);
            mini = std::min(mini, x);
        }
        double range = maxi - mini;
        if (range > maxrange) { bestdim = d; maxrange = range; }
    }
    // the value at the median position of the sorted coordinates (ties do not matter)
    std::vector<double> xs(N);
    for (int i = 0; i < N; i++) xs[i] = X[bestdim + (size_t)dim * dofs[i]];
    std::nth_element(xs.begin(), xs.begin() + N / 2, xs.end());
    double midv = xs[N / 2];
    for (int i = 0; i < N; i++) {
        int dof = dofs[i];
        invp[dof] = -1;
        for (int k = colptr[dof]; k < colptr[dof + 1]; k++) invp[rowval[k]] = -1;
    }
    for (int i = 0; i < N; i++) {
        int dof = dofs[i];
        invp[dof] = i;
        parts[i] = (X[bestdim + (size_t)dim * dof] < midv) ? 0 : 1;
    }
    for (int i = 0; i < N; i++) {
        int dof = dofs[i];
        if (parts[i] == 0) continue;
        for (int k = colptr[dof]; k < colptr[dof + 1]; k++) {
            int in = invp[rowval[k]];
            if (in == -1) continue;
            if (parts[in] == 0) { parts[i] = 2; break; }
        }
    }
}

// Modified nested dissection; partition.cpp:384-478 (geometric branch).
// partition.cpp:99-137: cut the widest coordinate at the value of the middle dof after
// sorting by it; dofs at or below go to part start, the others to start + 1
static void bissect_geo(const std::vector<int>& dofs, std::vector<int>& parts, const double* X, int dim, int start) {
    const int N = (int)dofs.size();
    if (N == 0) return;
    int bestdim = -1;
    double maxrange = -1.0;
    for (int d = 0; d < dim; d++) {
        double maxi = std::numeric_limits<double>::lowest(), mini = std::numeric_limits<double>::max();
        for (int idof : dofs) {
            maxi = std::max(maxi, X[d + (size_t)dim * idof]);
            mini = std::min(mini, X[d + (size_t)dim * idof]);
        }
        if (maxi - mini > maxrange) {
            bestdim = d;
            maxrange = maxi - mini;
        }
    }
    std::vector<int> tmp = dofs;
    std::sort(tmp.begin(), tmp.end(),
              [&](int i, int j) { return X[bestdim + (size_t)dim * i] < X[bestdim + (size_t)dim * j]; });
    const double midv = X[bestdim + (size_t)dim * tmp[N / 2]];
    for (int j : dofs) parts[j] = X[bestdim + (size_t)dim * j] <= midv ? start : start + 1;
}

// partition.cpp:245-285, geometric branch: nlevels - 1 rounds of bisection of every part
static std::vector<int> partition_RB(int N, int nlevels, const double* X, int dim) {
    std::vector<int> parts(N, 0);
    for (int depth = 0; depth < nlevels - 1; depth++) {
        const int np = 1 << depth;
        std::vector<std::vector<int>> dofs(np);
        for (int i = 0; i < N; i++) dofs[parts[i]].push_back(i);
        for (int k = 0; k < np; k++) bissect_geo(dofs[k], parts, X, dim, 2 * k);
    }
    return parts;
}

static std::vector<ClusterID> partition_modifiedND(const CSC& A, int nlevels, const double* X, int dim) {
    int N = A.n;
    // SpMat2CSC: the graph without self loops (partition.cpp:21-39)
    std::vector<int> colptr(N + 1, 0), rowval;
    for (int i = 0; i < N; i++) {
        colptr[i + 1] = colptr[i];
        for (int k = A.colptr[i]; k < A.colptr[i + 1]; k++) {
            int j = A.rowval[k];
            if (i != j) { rowval.push_back(j); colptr[i + 1]++; }
        }
    }
    std::vector<int> invp(N + 1), parttmp(N);
    std::vector<std::vector<int>> doms(1, std::vector<int>(N));
    std::iota(doms[0].begin(), doms[0].end(), 0);
    std::vector<ClusterID> part(N, ClusterID(SepID(nlevels - 1, 0), SepID(nlevels - 1, 0), SepID(nlevels - 1, 0)));
    for (int depth = 0; depth < nlevels - 1; depth++) {
        int level = nlevels - depth - 1;
        std::vector<std::vector<int>> newdoms((size_t)1 << (depth + 1));
        for (int sep = 0; sep < (1 << depth); sep++) {
            SepID idself(level, sep);
            std::vector<int> dofssep = doms[sep];
            std::sort(dofssep.begin(), dofssep.end());
            partition_nd_geo(colptr, rowval, dofssep, parttmp, X, dim, invp);
            SepID idleft(level - 1, 2 * sep), idright(level - 1, 2 * sep + 1);
            for (size_t i = 0; i < dofssep.size(); i++) {
                int j = dofssep[i];
                if (part[j].self == idself) {
                    if (parttmp[i] == 0) part[j].self = idleft;
                    else if (parttmp[i] == 1) part[j].self = idright;
                }
                if (parttmp[i] == 0) {
                    if (part[j].l == idself) part[j].l = idleft;
                    if (part[j].r == idself) part[j].r = idleft;
                } else if (parttmp[i] == 1) {
                    if (part[j].l == idself) part[j].l = idright;
                    if (part[j].r == idself) part[j].r = idright;
                } else if (parttmp[i] == 2) {
                    if (part[j].self == idself) { part[j].l = idleft; part[j].r = idright; }
                }
            }
            std::vector<int> newleft, newright;
            for (int i : dofssep) {
                const ClusterID& c = part[i];
                if (c.self == idleft || c.l == idleft || c.r == idleft) newleft.push_back(i);
                if (c.self == idright || c.l == idright || c.r == idright) newright.push_back(i);
            }
            newdoms[2 * sep] = newleft;
            newdoms[2 * sep + 1] = newright;
        }
        doms = newdoms;
    }
    return part;
}

// ---------------------------------------------------------------------------------
// Cluster / Edge (cluster.h:16-116, edge.h:32-44, cluster.cpp, edge.cpp)
// ---------------------------------------------------------------------------------
struct Cluster;
struct Edge {
    Cluster* n1;
    Cluster* n2;
    pMat A;  // rows n2->size, cols n1->size
    bool original;
};
using pEdge = std::unique_ptr<Edge>;

struct Cluster {
    int start, size, level, order;
    bool eliminated = false, sparsify;
    Cluster* parent = nullptr;
    std::vector<Cluster*> children;
    std::list<pEdge> edgesOut;   // pivot first
    std::list<Edge*> edgesIn;
    std::vector<double> x;       // x_ ; original_size() == x.size()
    pMat phi;                    // preserved vectors restricted to the cluster (size x nphi)
    Cluster(int st, int sz, int lv, int ord, bool sp) : start(st), size(sz), level(lv), order(ord), sparsify(sp) {
        reset_size(sz);
    }
    void reset_size(int s) { size = s; x.assign(s, 0.0); }
    int original_size() const { return (int)x.size(); }
    Edge* pivot() { return edgesOut.begin()->get(); }
    // cluster.cpp:113-123
    void add_edge(pEdge e) {
        if (e->n1 == e->n2) {
            edgesOut.push_front(std::move(e));
        } else {
            e->n2->edgesIn.push_back(e.get());
            edgesOut.push_back(std::move(e));
        }
    }
    // cluster.cpp:161-176 (std::list::sort is stable)
    void sort_edges() {
        edgesOut.sort([](const pEdge& a, const pEdge& b) {
            if (a->n1 == a->n2) return true;
            if (b->n1 == b->n2) return false;
            return a->n2->order < b->n2->order;
        });
        edgesIn.sort([](const Edge* a, const Edge* b) { return a->n1->order < b->n1->order; });
    }
    // cluster.cpp:32-45
    void set_eliminated() {
        for (auto& e : edgesOut) {
            Cluster* me = this;
            e->n2->edgesIn.remove_if([me](Edge* e2) { return e2->n1 == me; });
        }
        for (auto e : edgesIn) {
            Cluster* me = this;
            e->n1->edgesOut.remove_if([me](const pEdge& e2) { return e2->n2 == me; });
        }
        edgesIn.clear();
        edgesOut.clear();
        eliminated = true;
    }
    std::vector<Edge*> out_nbr() {
        std::vector<Edge*> r;
        auto it = edgesOut.begin();
        if (it != edgesOut.end()) ++it;
        for (; it != edgesOut.end(); ++it) r.push_back(it->get());
        return r;
    }
    std::vector<Edge*> out_all() {
        std::vector<Edge*> r;
        for (auto& e : edgesOut) r.push_back(e.get());
        return r;
    }
    std::vector<Edge*> in_nbr() { return std::vector<Edge*>(edgesIn.begin(), edgesIn.end()); }
};
using pCluster = std::unique_ptr<Cluster>;

// ---------------------------------------------------------------------------------
// Operations (operations.h:32-163, operations.cpp)
// ---------------------------------------------------------------------------------
enum OpKind {
    OP_SCALING_LLT = 0,
    OP_GEMM_SYMM_OUT = 1,
    OP_GEMM_SYMM_IN = 2,
    OP_ORTHOGONAL = 3,
    OP_MERGE = 4,
    OP_SPLIT = 5,
    OP_GEMM_OUT = 6,
    OP_GEMM_IN = 7,
    OP_SCALING_PLUQ = 8,
    OP_SCALING_LDLT = 9,
};

struct Op {
    OpKind kind;
    Cluster* self = nullptr;
    Cluster* nbr = nullptr;
    int ns = 0, nn = 0;          // Segment lengths captured at construction (head_x())
    pMat A;                      // LLT, Gemm block, v (Orthogonal), L (PLUQ)
    pMat U;                      // PLUQ
    std::vector<double> h;       // Orthogonal
    std::vector<int> p, q;       // PLUQ, LDLT (p)
    std::vector<double> s;       // LDLT: sign(D); Gemm ops of an LDLT pivot: the same signs
    int ilvl = 0;                // level at which the op was recorded

    long long nnz() const {
        switch (kind) {
            case OP_SCALING_LLT: return (long long)ns * (ns + 1) / 2;
            case OP_GEMM_SYMM_OUT: case OP_GEMM_SYMM_IN: case OP_GEMM_OUT: case OP_GEMM_IN:
                return (long long)ns * nn;
            case OP_ORTHOGONAL: return (long long)ns * ns;
            case OP_SCALING_PLUQ: return (long long)ns * ns + 2LL * ns;
            case OP_SCALING_LDLT: return (long long)ns * (ns + 1) / 2 + 2LL * ns;
            default: return 0;
        }
    }
    // self's x scaled by the signs (Gemm ops recorded with a diagonal, operations.cpp:55-93)
    std::vector<double> sx(const double* xs) const {
        std::vector<double> t(xs, xs + ns);
        for (int i = 0; i < ns; i++) t[i] *= s[i];
        return t;
    }
    void fwd() {
        double* xs = self ? self->x.data() : nullptr;
        switch (kind) {
            case OP_SCALING_LLT: trsv_lower(*A, xs, ns, false); break;
            case OP_GEMM_SYMM_OUT: case OP_GEMM_OUT:
                if (nn > 0 && ns > 0) {
                    if (s.empty()) gemv_sub(*A, false, xs, nbr->x.data());
                    else gemv_sub(*A, false, sx(xs).data(), nbr->x.data());
                }
                break;
            case OP_GEMM_SYMM_IN:
                if (nn > 0 && ns > 0) {
                    if (s.empty()) gemv_sub(*A, true, xs, nbr->x.data());
                    else gemv_sub(*A, true, sx(xs).data(), nbr->x.data());
                }
                break;
            case OP_SCALING_LDLT: {
                std::vector<double> t(ns);
                for (int i = 0; i < ns; i++) t[i] = xs[p[i]];
                std::copy(t.begin(), t.end(), xs);
                trsv_lower(*A, xs, ns, false);
                break;
            }
            case OP_GEMM_IN: break;
            case OP_ORTHOGONAL: ormqr_vec(*A, h, A->c, xs, true); break;
            case OP_MERGE: {
                int k = 0;
                for (auto c : self->children)
                    for (int i = 0; i < c->size; i++) self->x[k++] = c->x[i];
                break;
            }
            case OP_SPLIT: {
                Cluster* sib = nbr;
                for (int i = 0; i < sib->size; i++) sib->x[i] = self->x[self->size + i];
                break;
            }
            case OP_SCALING_PLUQ: {
                std::vector<double> t(ns);
                for (int i = 0; i < ns; i++) t[i] = xs[p[i]];
                std::copy(t.begin(), t.end(), xs);
                trsv_lower(*A, xs, ns, false);
                break;
            }
        }
    }
    // self -= s .* (op(A) nbr) (operations.cpp:65-73, 85-93)
    void sub_scaled(bool trans, double* xs) const {
        std::vector<double> t(ns, 0.0);
        gemv_sub(*A, trans, nbr->x.data(), t.data());  // t = -op(A) nbr
        for (int i = 0; i < ns; i++) xs[i] += s[i] * t[i];
    }
    void diag() {
        if (kind != OP_SCALING_LDLT) return;
        double* xs = self->x.data();
        for (int i = 0; i < ns; i++) xs[i] /= s[i];  // operations.cpp:139-141
    }
    void bwd() {
        double* xs = self ? self->x.data() : nullptr;
        switch (kind) {
            case OP_SCALING_LLT: trsv_lower(*A, xs, ns, true); break;
            case OP_GEMM_SYMM_OUT:
                if (nn > 0 && ns > 0) {
                    if (s.empty()) gemv_sub(*A, true, nbr->x.data(), xs);
                    else sub_scaled(true, xs);
                }
                break;
            case OP_GEMM_SYMM_IN: case OP_GEMM_IN:
                if (nn > 0 && ns > 0) {
                    if (s.empty() || kind == OP_GEMM_IN) gemv_sub(*A, false, nbr->x.data(), xs);
                    else sub_scaled(false, xs);
                }
                break;
            case OP_SCALING_LDLT: {
                trsv_lower(*A, xs, ns, true);
                std::vector<double> t(ns);
                for (int i = 0; i < ns; i++) t[p[i]] = xs[i];
                std::copy(t.begin(), t.end(), xs);
                break;
            }
            case OP_GEMM_OUT: break;
            case OP_ORTHOGONAL: ormqr_vec(*A, h, A->c, xs, false); break;
            case OP_MERGE: {
                int k = 0;
                for (auto c : self->children)
                    for (int i = 0; i < c->size; i++) c->x[i] = self->x[k++];
                break;
            }
            case OP_SPLIT: {
                Cluster* sib = nbr;
                for (int i = 0; i < sib->size; i++) self->x[self->size + i] = sib->x[i];
                break;
            }
            case OP_SCALING_PLUQ: {
                trsv_upper(*U, xs, ns);
                std::vector<double> t(ns);
                for (int i = 0; i < ns; i++) t[i] = xs[q[i]];
                std::copy(t.begin(), t.end(), xs);
                break;
            }
        }
    }
};
using pOp = std::unique_ptr<Op>;

// ---------------------------------------------------------------------------------
// Per-level log and flop log (util.h:262-401)
// ---------------------------------------------------------------------------------
struct IStats {
    long long sum = 0;
    int count = 0, mn = INT32_MAX, mx = INT32_MIN;
    void add(int v) { sum += v; count++; mn = std::min(mn, v); mx = std::max(mx, v); }
};
struct LevelLog {
    int dofs_nd = 0, dofs_left_nd = 0, dofs_left_elim = 0, dofs_left_spars = 0;
    long long fact_nnz = 0;
    IStats rank_before, rank_after, nbrs;
    int ignored = 0;
    double t_elim = 0, t_scale = 0, t_spars = 0, t_merge = 0;
    double flops_potf = 0, flops_trsm = 0, flops_gemm = 0, flops_geqp3 = 0;
};

enum SymmKind { SPD = 0, SYM = 1, GEN = 2 };
enum ScalingKind { S_LLT = 0, S_PLU = 3, S_PLUQ = 4, S_LDLT = 5 };

// ---------------------------------------------------------------------------------
// Tree (tree.h, tree.cpp)
// ---------------------------------------------------------------------------------
struct Tree {
    bool verb = false;
    bool geo = false;
    int ilvl = 0;
    int nlevels;
    double tol = 10.0;       // tree.cpp:94
    int skip = 0;
    int symm = SPD;
    int scale_kind = S_LLT;
    bool use_want_sparsify = true;
    // preservation (tree.h:57, 140-141): the columns of phi (N x nphi, natural ordering,
    // column-major) are kept in the range of every sparsification
    bool preserve = false;
    std::vector<double> phi;
    int nphi = 0;
    const double* X = nullptr;
    int dim = 0;
    int max_order = 0;
    std::vector<int> perm;
    std::list<pOp> ops;
    int current_bottom = 0;
    std::vector<std::list<pCluster>> bottoms;
    std::vector<pCluster> others;
    std::vector<LevelLog> log;
    std::vector<ClusterID> part;  // natural ordering
    double t_partition = 0, t_assemble = 0, t_factorize = 0;
    // ranks for parity: (level, cluster order, rows, rank) of every sparsified cluster
    std::vector<std::array<int, 4>> rank_log;

    explicit Tree(int nl) : nlevels(nl), bottoms(nl), log(nl) {}
    bool symmetry() const { return symm == SPD || symm == SYM; }
    int get_new_order() { return max_order++; }
    std::list<pCluster>& bottom_current() { return bottoms[current_bottom]; }
    std::list<pCluster>& bottom_original() { return bottoms[0]; }
    int N() const { return (int)perm.size(); }

    int ndofs_left() {
        int n = 0;
        for (auto& s : bottom_current())
            if (!s->eliminated) n += s->size;
        return n;
    }
    int nclusters_left() {
        int n = 0;
        for (auto& s : bottom_current())
            if (!s->eliminated) n++;
        return n;
    }
    long long nnz() const {
        long long n = 0;
        for (auto& op : ops) n += op->nnz();
        return n;
    }
    int get_stop() const {  // tree.cpp:158-169
        int stop = (int)perm.size();
        for (auto& l : log) {
            if (l.dofs_left_elim > 0) stop = std::min(stop, l.dofs_left_elim);
            if (l.dofs_left_spars > 0) stop = std::min(stop, l.dofs_left_spars);
        }
        return stop;
    }

    // tree.cpp:306-419
    void partition(const CSC& A) {
        double t0 = now_s();
        int N = A.n;
        if (geo) {
            part = partition_modifiedND(A, nlevels, X, dim);
        } else {
            throw std::runtime_error("oracle: algebraic (METIS) ordering is not restated; set geometry");
        }
        for (int i = 0; i < N; i++) log[part[i].self.lvl].dofs_nd += 1;
        log[nlevels - 1].dofs_left_nd = 0;
        for (int l = nlevels - 2; l >= 0; l--) log[l].dofs_left_nd = log[l + 1].dofs_nd + log[l + 1].dofs_left_nd;
        perm.resize(N);
        std::iota(perm.begin(), perm.end(), 0);
        std::vector<ClusterID> pm = part;
        auto cmp = [&pm](int i, int j) { return pm[i] < pm[j]; };
        std::stable_sort(perm.begin(), perm.end(), cmp);
        for (int lvl = 1; lvl < nlevels; lvl++) {
            for (auto& c : pm) c = merge_if(c, lvl);
            std::stable_sort(perm.begin(), perm.end(), cmp);
        }
        std::map<Cluster*, ClusterID> ids;
        for (int k = 0; k < N;) {
            int knext = k + 1;
            ClusterID id = part[perm[k]];
            while (knext < N && part[perm[knext]] == id) knext++;
            auto self = std::make_unique<Cluster>(k, knext - k, id.self.lvl, get_new_order(), id.l.lvl == 0 && id.r.lvl == 0);
            ids[self.get()] = id;
            bottoms[0].push_back(std::move(self));
            k = knext;
        }
        for (int lvl = 1; lvl < nlevels; lvl++) {
            auto begin = std::find_if(bottoms[lvl - 1].begin(), bottoms[lvl - 1].end(),
                                      [lvl](const pCluster& s) { return s->level >= lvl; });
            auto end = bottoms[lvl - 1].end();
            std::map<Cluster*, ClusterID> pids;
            for (auto it = begin; it != end; ++it) pids[it->get()] = merge_if(ids.at(it->get()), lvl);
            for (auto k = begin; k != end;) {
                ClusterID idp = pids.at(k->get());
                std::vector<Cluster*> ch;
                ch.push_back(k->get());
                int cstart = (*k)->start, csize = (*k)->size;
                ++k;
                while (k != end && idp == pids.at(k->get())) {
                    ch.push_back(k->get());
                    csize += (*k)->size;
                    ++k;
                }
                auto parent = std::make_unique<Cluster>(cstart, csize, idp.self.lvl, get_new_order(),
                                                        idp.l.lvl == lvl && idp.r.lvl == lvl);
                for (auto c : ch) { c->parent = parent.get(); parent->children.push_back(c); }
                ids[parent.get()] = idp;
                bottoms[lvl].push_back(std::move(parent));
            }
        }
        t_partition = now_s() - t0;
    }

    // LoRaSp ordering (tree.cpp:421-503): recursive bisection; every cluster sits at the top
    // level (none is eliminated as an interior), pairs of consecutive clusters merge
    std::vector<int> rb_parts;  // natural ordering
    bool lorasp = false;
    void partition_lorasp(const CSC& A) {
        double t0 = now_s();
        const int N = A.n;
        if (!geo) throw std::runtime_error("oracle: algebraic (METIS) ordering is not restated; set geometry");
        rb_parts = partition_RB(N, nlevels, X, dim);
        const std::vector<int>& parts = rb_parts;
        perm.resize(N);
        std::iota(perm.begin(), perm.end(), 0);
        std::sort(perm.begin(), perm.end(), [&parts](int i, int j) { return parts[i] < parts[j]; });
        std::map<Cluster*, int> cid;
        const int lvltop = nlevels - 1;
        for (int k = 0; k < N;) {
            int knext = k + 1;
            const int id = parts[perm[k]];
            while (knext < N && parts[perm[knext]] == id) knext++;
            auto self = std::make_unique<Cluster>(k, knext - k, lvltop, get_new_order(), true);
            cid[self.get()] = self->order;
            bottoms[0].push_back(std::move(self));
            k = knext;
        }
        for (int lvl = 1; lvl < nlevels; lvl++) {
            auto k = bottoms[lvl - 1].begin();
            const auto end = bottoms[lvl - 1].end();
            while (k != end) {
                const int idp = cid.at(k->get()) / 2;
                std::vector<Cluster*> ch{k->get()};
                int cstart = (*k)->start, csize = (*k)->size;
                ++k;
                while (k != end && cid.at(k->get()) / 2 == idp) {
                    ch.push_back(k->get());
                    csize += (*k)->size;
                    ++k;
                }
                auto parent = std::make_unique<Cluster>(cstart, csize, lvltop, get_new_order(), true);
                for (auto c : ch) { c->parent = parent.get(); parent->children.push_back(c); }
                cid[parent.get()] = idp;
                bottoms[lvl].push_back(std::move(parent));
            }
        }
        lorasp = true;
        t_partition = now_s() - t0;
    }

    // tree.cpp:505-575
    void assemble(const CSC& A) {
        double t0 = now_s();
        int N = this->N();
        CSC App = symm_perm(A, perm);
        std::vector<Cluster*> cmap(N);
        for (auto& s : bottom_original())
            for (int k = s->start; k < s->start + s->size; k++) cmap[k] = s.get();
        for (auto& sp : bottom_original()) {
            Cluster* self = sp.get();
            std::set<int> nbr_orders;
            std::map<int, Cluster*> by_order;
            for (int j = self->start; j < self->start + self->size; j++) {
                for (int k = App.colptr[j]; k < App.colptr[j + 1]; k++) {
                    int row = App.rowval[k];
                    if (symmetry() && row < j) continue;
                    Cluster* n = cmap[row];
                    nbr_orders.insert(n->order);
                    by_order[n->order] = n;
                }
            }
            nbr_orders.insert(self->order);
            by_order[self->order] = self;
            for (int o : nbr_orders) {
                Cluster* nbr = by_order[o];
                auto M = std::make_unique<Mat>(nbr->size, self->size);
                // block2dense (util.cpp:454-486)
                for (int col = 0; col < self->size; col++) {
                    int j = self->start + col;
                    for (int k = App.colptr[j]; k < App.colptr[j + 1]; k++) {
                        int row = App.rowval[k];
                        if (row >= nbr->start && row < nbr->start + nbr->size) (*M)(row - nbr->start, col) = App.val[k];
                    }
                }
                self->add_edge(std::make_unique<Edge>(Edge{self, nbr, std::move(M), true}));
            }
            self->sort_edges();
        }
        t_assemble = now_s() - t0;
    }

    // ---- elimination kernels ----------------------------------------------------
    void potf_cluster(Cluster* self) {  // tree.cpp:582-593
        Mat* Ass = self->pivot()->A.get();
        int info = potf(*Ass);
        if (info != 0) throw std::runtime_error("Error: Non-SPD Pivot");
        double n = Ass->r;
        log[ilvl].flops_potf += n * n * n / 3.0;
    }
    void getf_cluster(Cluster* self, pMat& L, pMat& U, std::vector<int>& p, std::vector<int>& q) {  // tree.cpp:614-635
        Mat* Ass = self->pivot()->A.get();
        if (scale_kind == S_PLUQ) throw std::runtime_error("oracle: PLUQ (full pivoting) is not restated");
        int info = getf(*Ass, p);
        if (info != 0) throw std::runtime_error("Error: Singular Pivot");
        q.resize(self->size);
        std::iota(q.begin(), q.end(), 0);
        L = std::make_unique<Mat>();
        U = std::make_unique<Mat>();
        split_LU(*Ass, *L, *U);
        double n = Ass->r;
        log[ilvl].flops_potf += 2.0 * n * n * n / 3.0;
    }
    void panel_potf(Cluster* self) {  // tree.cpp:717-724, 640-663
        Mat& L = *self->pivot()->A;
        for (auto e : self->in_nbr()) {
            trsm_left_lower(L, *e->A);
            log[ilvl].flops_trsm += (double)e->A->c * e->A->r * e->A->r;
        }
        for (auto e : self->out_nbr()) {
            trsm_right_lower_trans(L, *e->A);
            log[ilvl].flops_trsm += (double)e->A->r * e->A->c * e->A->c;
        }
    }
    void panel_getf(Cluster* self, Mat& L, Mat& U, std::vector<int>& p) {  // tree.cpp:668-689, 735-742
        for (auto e : self->in_nbr()) {
            Mat& Asn = *e->A;
            Mat T(Asn.r, Asn.c);
            for (int j = 0; j < Asn.c; j++)
                for (int i = 0; i < Asn.r; i++) T(i, j) = Asn(p[i], j);
            Asn = std::move(T);
            trsm_left_lower(L, Asn);
            log[ilvl].flops_trsm += (double)Asn.c * Asn.r * Asn.r;
        }
        for (auto e : self->out_nbr()) {
            // q is the identity for PLU
            trsm_right_upper(U, *e->A);
            log[ilvl].flops_trsm += (double)e->A->r * e->A->c * e->A->c;
        }
    }
    // tree.cpp:748-793; with diag (LDLT): C -= op(A1) diag^-1 op(A2) on the whole block
    void gemm_edges(Edge* e1, Edge* e2, bool t1, bool t2, const std::vector<double>* diag = nullptr) {
        Cluster* s = t1 ? e1->n2 : e1->n1;
        Cluster* n1 = t1 ? e1->n1 : e1->n2;
        Cluster* n2 = t2 ? e2->n2 : e2->n1;
        Edge* found = nullptr;
        for (auto& e : n2->edgesOut)
            if (e->n2 == n1) { found = e.get(); break; }
        if (!found) {
            n2->add_edge(std::make_unique<Edge>(Edge{n2, n1, std::make_unique<Mat>(n1->size, n2->size), false}));
            for (auto& e : n2->edgesOut)
                if (e->n2 == n1) { found = e.get(); break; }
        }
        Mat& C = *found->A;
        if (diag) {
            Mat B = *e2->A;  // op(B) has the s rows: rows of B, or columns when t2
            for (int j = 0; j < B.c; j++)
                for (int i = 0; i < B.r; i++) B(i, j) /= (*diag)[t2 ? j : i];
            gemm_sub(*e1->A, t1, B, t2, C);
            log[ilvl].flops_gemm += 2.0 * C.r * C.c * s->size;
        } else if (n1 == n2 && symmetry()) {
            syrk_sub_lower(*e1->A, t1, C);
            log[ilvl].flops_gemm += (double)C.r * C.r * s->size;
        } else {
            gemm_sub(*e1->A, t1, *e2->A, t2, C);
            log[ilvl].flops_gemm += 2.0 * C.r * C.c * s->size;
        }
    }
    void schur_symmetric(Cluster* self, const std::vector<double>* diag = nullptr) {  // tree.cpp:862-883
        auto outs = self->out_nbr();
        auto ins = self->in_nbr();
        for (auto e1 : outs)
            for (auto e2 : outs)
                if (e1->n2->order >= e2->n2->order) gemm_edges(e1, e2, false, true, diag);
        for (auto e1 : ins)
            for (auto e2 : ins)
                if (e1->n1->order >= e2->n1->order) gemm_edges(e1, e2, true, false, diag);
        for (auto e1 : outs)
            for (auto e2 : ins) gemm_edges(e1, e2, false, false, diag);
    }
    // tree.cpp:596-611
    void ldlt_cluster(Cluster* self, Mat& L, std::vector<double>& s, std::vector<int>& p) {
        const Mat& Ass = *self->pivot()->A;
        if (ldlt(Ass, L, s, p) != 0) throw std::runtime_error("Error: Singular Pivot");
        double n = Ass.r;
        log[ilvl].flops_potf += n * n * n / 3.0;
    }
    // tree.cpp:691-715, 726-733: A_sn <- L^-1 P^T A_sn (in-edges), A_ns <- A_ns P L^-T (out-edges)
    void panel_ldlt(Cluster* self, const Mat& L, const std::vector<int>& p) {
        for (auto e : self->in_nbr()) {
            Mat& Asn = *e->A;
            Mat T(Asn.r, Asn.c);
            for (int j = 0; j < Asn.c; j++)
                for (int i = 0; i < Asn.r; i++) T(i, j) = Asn(p[i], j);
            Asn = std::move(T);
            trsm_left_lower(L, Asn);
            log[ilvl].flops_trsm += (double)Asn.c * Asn.r * Asn.r;
        }
        for (auto e : self->out_nbr()) {
            Mat& Ans = *e->A;
            Mat T(Ans.r, Ans.c);
            for (int j = 0; j < Ans.c; j++)
                for (int i = 0; i < Ans.r; i++) T(i, j) = Ans(i, p[j]);
            Ans = std::move(T);
            trsm_right_lower_trans(L, Ans);
            log[ilvl].flops_trsm += (double)Ans.r * Ans.c * Ans.c;
        }
    }
    void push_op(pOp op) { op->ilvl = ilvl; ops.push_back(std::move(op)); }
    pOp make_op(OpKind k, Cluster* self, Cluster* nbr, pMat A) {
        auto op = std::make_unique<Op>();
        op->kind = k;
        op->self = self;
        op->nbr = nbr;
        op->ns = self ? self->size : 0;
        op->nn = nbr ? nbr->size : 0;
        op->A = std::move(A);
        return op;
    }
    // tree.cpp:895-967
    void eliminate_cluster(Cluster* self) {
        if (scale_kind == S_LLT) {
            potf_cluster(self);
            panel_potf(self);
            schur_symmetric(self);
            push_op(make_op(OP_SCALING_LLT, self, nullptr, std::move(self->pivot()->A)));
            for (auto e : self->out_nbr()) push_op(make_op(OP_GEMM_SYMM_OUT, self, e->n2, std::move(e->A)));
            for (auto e : self->in_nbr()) push_op(make_op(OP_GEMM_SYMM_IN, self, e->n1, std::move(e->A)));
        } else if (scale_kind == S_LDLT) {  // tree.cpp:911-928
            auto L = std::make_unique<Mat>();
            std::vector<double> s;
            std::vector<int> p;
            ldlt_cluster(self, *L, s, p);
            panel_ldlt(self, *L, p);
            schur_symmetric(self, &s);
            auto op = make_op(OP_SCALING_LDLT, self, nullptr, std::move(L));
            op->s = s;
            op->p = p;
            push_op(std::move(op));
            for (auto e : self->out_nbr()) {
                auto g = make_op(OP_GEMM_SYMM_OUT, self, e->n2, std::move(e->A));
                g->s = s;
                push_op(std::move(g));
            }
            for (auto e : self->in_nbr()) {
                auto g = make_op(OP_GEMM_SYMM_IN, self, e->n1, std::move(e->A));
                g->s = s;
                push_op(std::move(g));
            }
        } else if (scale_kind == S_PLU || scale_kind == S_PLUQ) {
            pMat L, U;
            std::vector<int> p, q;
            getf_cluster(self, L, U, p, q);
            panel_getf(self, *L, *U, p);
            for (auto e1 : self->out_nbr())
                for (auto e2 : self->in_nbr()) gemm_edges(e1, e2, false, false);
            auto op = make_op(OP_SCALING_PLUQ, self, nullptr, std::move(L));
            op->U = std::move(U);
            op->p = p;
            op->q = q;
            push_op(std::move(op));
            for (auto e : self->out_nbr()) push_op(make_op(OP_GEMM_OUT, self, e->n2, std::move(e->A)));
            for (auto e : self->in_nbr()) push_op(make_op(OP_GEMM_IN, self, e->n1, std::move(e->A)));
        } else {
            throw std::runtime_error("oracle: scaling kind not restated");
        }
        self->set_eliminated();
    }
    // tree.cpp:796-856
    void scale_cluster(Cluster* self) {
        if (scale_kind == S_LLT) {
            potf_cluster(self);
            panel_potf(self);
            if (preserve) trmm_trans(*self->pivot()->A, *self->phi);  // tree.cpp:807-809
            push_op(make_op(OP_SCALING_LLT, self, nullptr, std::move(self->pivot()->A)));
        } else if (scale_kind == S_LDLT) {  // tree.cpp:812-830: the new pivot is diag(sign D)
            auto L = std::make_unique<Mat>();
            std::vector<double> s;
            std::vector<int> p;
            ldlt_cluster(self, *L, s, p);
            panel_ldlt(self, *L, p);
            if (preserve) {  // tree.cpp:824-827: phi <- L^T P^T phi
                Mat& F = *self->phi;
                Mat T(F.r, F.c);
                for (int j = 0; j < F.c; j++)
                    for (int i = 0; i < F.r; i++) T(i, j) = F(p[i], j);
                F = std::move(T);
                trmm_trans(*L, F);
            }
            auto op = make_op(OP_SCALING_LDLT, self, nullptr, std::move(L));
            op->s = s;
            op->p = p;
            push_op(std::move(op));
            auto D = std::make_unique<Mat>(self->size, self->size);
            for (int i = 0; i < self->size; i++) (*D)(i, i) = s[i];
            self->pivot()->A = std::move(D);
            return;
        } else {
            pMat L, U;
            std::vector<int> p, q;
            getf_cluster(self, L, U, p, q);
            panel_getf(self, *L, *U, p);
            auto op = make_op(OP_SCALING_PLUQ, self, nullptr, std::move(L));
            op->U = std::move(U);
            op->p = p;
            op->q = q;
            push_op(std::move(op));
        }
        self->pivot()->A = std::make_unique<Mat>(Mat::eye(self->size));
    }

    // ---- sparsification ---------------------------------------------------------
    // tree.cpp:1189-1224 (pred == true)
    pMat assemble_Asn(Cluster* self) {
        int rows = self->size, cols = 0;
        auto ins = self->in_nbr();
        auto outs = self->out_nbr();
        for (auto e : ins) cols += e->n1->size;
        for (auto e : outs) cols += e->n2->size;
        auto Asn = std::make_unique<Mat>(rows, cols);
        int c = 0;
        for (auto e : ins) {
            for (int j = 0; j < e->n1->size; j++)
                for (int i = 0; i < rows; i++) (*Asn)(i, c + j) = (*e->A)(i, j);
            c += e->n1->size;
        }
        for (auto e : outs) {
            for (int j = 0; j < e->n2->size; j++)
                for (int i = 0; i < rows; i++) (*Asn)(i, c + j) = (*e->A)(j, i);
            c += e->n2->size;
        }
        log[ilvl].nbrs.add(cols);
        return Asn;
    }
    // tree.cpp:980-1104 (pred == true branch).  Pivot I (SPD, GEN), or (SYM) the signs of
    // the scaling, transformed to Q^T piv Q and split: the sibling's pivot, an edge
    // original -> sibling, and the original's new pivot (tree.cpp:1069-1097).
    // AsnP == nullptr: the preservation branch (pred == false, keep_sibling == false):
    // phi and every edge block get Q^T (in-edges and phi from the left, out-edges from the
    // right) and keep their first osize rows / columns; the sibling gets no edge.
    // farfield (LoRaSp, tree.cpp:1411-1415: pred = !original, keep_sibling == true): the
    // fill-in edges take AsnP, the original ones get Q^T and hand their last rows /
    // columns to a new edge neighbour -> sibling (tree.cpp:1018-1064).
    Cluster* shrink_split(Cluster* original, int osize, Mat* AsnP, const Mat& v, const std::vector<double>& h,
                          bool farfield = false) {
        const int n0 = original->size;
        int sib_size = original->size - osize;
        auto psib = std::make_unique<Cluster>(original->start + osize, sib_size, original->level, get_new_order(),
                                              original->sparsify);
        Cluster* sib = psib.get();
        original->size = osize;  // set_size keeps x
        const int k = (int)h.size();
        auto qt_rows = [&](Mat& B) {  // B (n0 x c) <- (Q^T B)[0:osize, :]
            for (int j = 0; j < B.c; j++) ormqr_vec(v, h, k, B.col(j), true);
            Mat T(osize, B.c);
            for (int j = 0; j < B.c; j++)
                for (int i = 0; i < osize; i++) T(i, j) = B(i, j);
            B = std::move(T);
        };
        if (preserve) qt_rows(*original->phi);  // tree.cpp:993-1002
        int col = 0;
        auto keep_tail = [&](Cluster* n, const Mat& Qt, bool orig) {  // Qt: n0 x n, rows osize.. -> sibling
            auto S = std::make_unique<Mat>(sib_size, Qt.c);
            for (int j = 0; j < Qt.c; j++)
                for (int i = 0; i < sib_size; i++) (*S)(i, j) = Qt(osize + i, j);
            n->add_edge(std::make_unique<Edge>(Edge{n, sib, std::move(S), orig}));
        };
        for (auto e : original->in_nbr()) {
            int cols = e->n1->size;
            if (farfield && e->original) {
                Mat& B = *e->A;
                for (int j = 0; j < B.c; j++) ormqr_vec(v, h, k, B.col(j), true);
                keep_tail(e->n1, B, true);
                Mat T(osize, B.c);
                for (int j = 0; j < B.c; j++)
                    for (int i = 0; i < osize; i++) T(i, j) = B(i, j);
                B = std::move(T);
                continue;
            }
            if (!AsnP) {
                qt_rows(*e->A);
                continue;
            }
            auto M = std::make_unique<Mat>(osize, cols);
            for (int j = 0; j < cols; j++)
                for (int i = 0; i < osize; i++) (*M)(i, j) = (*AsnP)(i, col + j);
            e->A = std::move(M);
            col += cols;
        }
        for (auto e : original->out_nbr()) {
            int cols = e->n2->size;
            if (farfield && e->original) {  // A Q, row by row as Q^T A^T
                Mat& B = *e->A;
                Mat Bt(B.c, B.r);
                for (int j = 0; j < B.c; j++)
                    for (int i = 0; i < B.r; i++) Bt(j, i) = B(i, j);
                for (int j = 0; j < Bt.c; j++) ormqr_vec(v, h, k, Bt.col(j), true);
                keep_tail(e->n2, Bt, true);
                Mat M(B.r, osize);
                for (int j = 0; j < osize; j++)
                    for (int i = 0; i < B.r; i++) M(i, j) = Bt(j, i);
                B = std::move(M);
                continue;
            }
            if (!AsnP) {  // A Q, row by row as Q^T A^T
                Mat& B = *e->A;
                Mat Bt(B.c, B.r);
                for (int j = 0; j < B.c; j++)
                    for (int i = 0; i < B.r; i++) Bt(j, i) = B(i, j);
                qt_rows(Bt);
                Mat M(B.r, osize);
                for (int j = 0; j < osize; j++)
                    for (int i = 0; i < B.r; i++) M(i, j) = Bt(j, i);
                B = std::move(M);
                continue;
            }
            auto M = std::make_unique<Mat>(cols, osize);
            for (int j = 0; j < cols; j++)
                for (int i = 0; i < osize; i++) (*M)(j, i) = (*AsnP)(i, col + j);
            e->A = std::move(M);
            col += cols;
        }
        if (symm != SYM) {
            // pivot is identity: Aoo = I_osize, Ass = I_sib
            sib->add_edge(std::make_unique<Edge>(Edge{sib, sib, std::make_unique<Mat>(Mat::eye(sib_size)), true}));
            original->pivot()->A = std::make_unique<Mat>(Mat::eye(osize));
        } else {
            Mat& piv = *original->pivot()->A;  // n0 x n0, the signs of the scaling
            const int k = (int)h.size();
            // Deviation: when every sign is the same, Q^T D Q = D exactly and is kept as it
            // is; the reference forms it in floating point, where its zero entries become
            // rounding noise whose signs then steer later Householder reflectors.
            bool uniform = true;
            for (int i = 1; i < n0; i++) uniform = uniform && piv(i, i) == piv(0, 0);
            std::vector<double> t(n0);
            for (int r = 0; r < n0 && !uniform; r++) {  // piv <- piv Q (row by row: Q^T row^T)
                for (int c = 0; c < n0; c++) t[c] = piv(r, c);
                ormqr_vec(v, h, k, t.data(), true);
                for (int c = 0; c < n0; c++) piv(r, c) = t[c];
            }
            for (int c = 0; c < n0 && !uniform; c++) ormqr_vec(v, h, k, &piv(0, c), true);  // piv <- Q^T piv
            auto Aoo = std::make_unique<Mat>(osize, osize);
            auto Ass = std::make_unique<Mat>(sib_size, sib_size);
            auto Aso = std::make_unique<Mat>(sib_size, osize);
            for (int j = 0; j < osize; j++)
                for (int i = 0; i < osize; i++) (*Aoo)(i, j) = piv(i, j);
            for (int j = 0; j < sib_size; j++)
                for (int i = 0; i < sib_size; i++) (*Ass)(i, j) = piv(osize + i, osize + j);
            for (int j = 0; j < osize; j++)
                for (int i = 0; i < sib_size; i++) (*Aso)(i, j) = piv(osize + i, j);
            sib->add_edge(std::make_unique<Edge>(Edge{sib, sib, std::move(Ass), true}));
            original->add_edge(std::make_unique<Edge>(Edge{original, sib, std::move(Aso), true}));
            original->pivot()->A = std::move(Aoo);
        }
        others.push_back(std::move(psib));
        push_op(make_op(OP_SPLIT, original, sib, nullptr));
        return sib;
    }
    // tree.cpp:1292-1347
    void sparsify_adaptive_only(Cluster* self) {
        auto Asn = assemble_Asn(self);
        int rows = Asn->r, cols = Asn->c;
        std::vector<int> jpvt;
        std::vector<double> ht;
        geqp3(*Asn, jpvt, ht);
        std::vector<double> diag(std::min(rows, cols));
        for (size_t i = 0; i < diag.size(); i++) diag[i] = (*Asn)((int)i, (int)i);
        int rank = choose_rank(diag, tol);
        rank_log.push_back({ilvl, self->order, rows, rank});
        {
            double m = rows, n = cols, k = std::min(rank, (int)diag.size());
            log[ilvl].flops_geqp3 += 4.0 * m * n * k - 2.0 * k * k * (m + n) + 4.0 * k * k * k / 3.0;
        }
        if (rank >= rows) return;
        auto v = std::make_unique<Mat>(rows, rank);
        for (int j = 0; j < rank; j++)
            for (int i = 0; i < rows; i++) (*v)(i, j) = (*Asn)(i, j);
        auto op = make_op(OP_ORTHOGONAL, self, nullptr, std::move(v));
        op->h.assign(ht.begin(), ht.begin() + rank);
        const Op* qop = op.get();
        push_op(std::move(op));
        // AsnP = triu(R[:rank,:]) P^T : column jpvt[j] of AsnP is column j of triu(R)
        Mat AsnP(rank, cols);
        for (int j = 0; j < cols; j++)
            for (int i = 0; i < rank && i <= j; i++) AsnP(i, jpvt[j]) = (*Asn)(i, j);
        Cluster* sib = shrink_split(self, rank, &AsnP, *qop->A, qop->h);
        eliminate_cluster(sib);
    }
    // tree.cpp:1226-1254: [A_sn phi_n (in-edges) | A_ns^T phi_n (out-edges, pivot first)]
    pMat assemble_Asphi(Cluster* self) {
        const int rows = self->size;
        auto ins = self->in_nbr();
        auto outs = self->out_all();
        auto M = std::make_unique<Mat>(rows, nphi * (int)(ins.size() + outs.size()));
        int c = 0;
        for (auto e : ins) {  // A (rows x n) phi_n (n x nphi)
            const Mat& A = *e->A;
            const Mat& F = *e->n1->phi;
            for (int q = 0; q < nphi; q++, c++)
                for (int i = 0; i < rows; i++) {
                    double s = 0.0;
                    for (int kk = 0; kk < A.c; kk++) s += A(i, kk) * F(kk, q);
                    (*M)(i, c) = s;
                }
        }
        for (auto e : outs) {  // A^T (A: n x rows) phi_n
            const Mat& A = *e->A;
            const Mat& F = *e->n2->phi;
            for (int q = 0; q < nphi; q++, c++)
                for (int i = 0; i < rows; i++) {
                    double s = 0.0;
                    for (int kk = 0; kk < A.r; kk++) s += A(kk, i) * F(kk, q);
                    (*M)(i, c) = s;
                }
        }
        return M;
    }
    void record_q_and_split(Cluster* self, pMat v, std::vector<double> h) {
        const int rank = (int)h.size();
        auto op = make_op(OP_ORTHOGONAL, self, nullptr, std::move(v));
        op->h = std::move(h);
        const Op* qop = op.get();
        push_op(std::move(op));
        Cluster* sib = shrink_split(self, rank, nullptr, *qop->A, qop->h);
        eliminate_cluster(sib);
    }
    // tree.cpp:1257-1287: Q from the QR of [A_sn phi, phi]; rank = its column count
    void sparsify_preserve_only(Cluster* self) {
        auto A = assemble_Asphi(self);
        const int rows = A->r, cols = A->c;
        if (cols >= rows) {
            rank_log.push_back({ilvl, self->order, rows, rows});
            return;
        }
        std::vector<double> h;
        geqrf(*A, h);
        rank_log.push_back({ilvl, self->order, rows, cols});
        record_q_and_split(self, std::move(A), std::move(h));
    }
    // tree.cpp:1350-1409: Q1 spans [A_sn phi, phi]; the QRCP of (I - Q1 Q1^T) Asn truncated
    // at tol gives Q2; Q from the QR of [Q1 Q2]
    void sparsify_preserve_adaptive(Cluster* self) {
        const int rows = self->size;
        auto Q1 = assemble_Asphi(self);
        const int rank1 = std::min(rows, Q1->c);
        std::vector<double> h1;
        geqrf(*Q1, h1);
        Q1->c = rank1;
        Q1->v.resize((size_t)rows * rank1);
        orgqr(*Q1, h1);
        auto Asn = assemble_Asn(self);
        const int cols2 = Asn->c;
        {  // Asn -= Q1 (Q1^T Asn)
            std::vector<double> w(rank1);
            for (int j = 0; j < cols2; j++) {
                double* a = Asn->col(j);
                for (int q = 0; q < rank1; q++) {
                    double s = 0.0;
                    for (int i = 0; i < rows; i++) s += Q1->col(q)[i] * a[i];
                    w[q] = s;
                }
                for (int i = 0; i < rows; i++) {
                    double s = 0.0;
                    for (int q = 0; q < rank1; q++) s += Q1->col(q)[i] * w[q];
                    a[i] -= s;
                }
            }
        }
        std::vector<int> jpvt;
        std::vector<double> h2;
        geqp3(*Asn, jpvt, h2);
        std::vector<double> diag(std::min(rows, cols2));
        for (size_t i = 0; i < diag.size(); i++) diag[i] = (*Asn)((int)i, (int)i);
        const int rank2 = choose_rank(diag, tol);
        const int rank = rank1 + rank2;
        if (rank >= rows) {
            rank_log.push_back({ilvl, self->order, rows, rows});
            return;
        }
        Mat Q2(rows, rank2);
        for (int j = 0; j < rank2; j++)
            for (int i = 0; i < rows; i++) Q2(i, j) = (*Asn)(i, j);
        h2.resize(rank2);
        orgqr(Q2, h2);
        auto V = std::make_unique<Mat>(rows, rank);
        for (int j = 0; j < rank1; j++)
            for (int i = 0; i < rows; i++) (*V)(i, j) = (*Q1)(i, j);
        for (int j = 0; j < rank2; j++)
            for (int i = 0; i < rows; i++) (*V)(i, rank1 + j) = Q2(i, j);
        std::vector<double> h;
        geqrf(*V, h);
        rank_log.push_back({ilvl, self->order, rows, rank});
        record_q_and_split(self, std::move(V), std::move(h));
    }
    // LoRaSp sparsification (tree.cpp:1292-1347 with pred = !original, tree.cpp:1411-1415):
    // the QRCP sees only the fill-in edges; the original edges keep their coupling to the
    // sibling, whose elimination then updates the cluster's neighbours
    void sparsify_farfield(Cluster* self) {
        const int rows = self->size;
        std::vector<Edge*> ins, outs;
        for (auto e : self->in_nbr())
            if (!e->original) ins.push_back(e);
        for (auto e : self->out_nbr())
            if (!e->original) outs.push_back(e);
        int cols = 0;
        for (auto e : ins) cols += e->n1->size;
        for (auto e : outs) cols += e->n2->size;
        Mat Asn(rows, cols);
        int c = 0;
        for (auto e : ins) {
            for (int j = 0; j < e->n1->size; j++)
                for (int i = 0; i < rows; i++) Asn(i, c + j) = (*e->A)(i, j);
            c += e->n1->size;
        }
        for (auto e : outs) {
            for (int j = 0; j < e->n2->size; j++)
                for (int i = 0; i < rows; i++) Asn(i, c + j) = (*e->A)(j, i);
            c += e->n2->size;
        }
        log[ilvl].nbrs.add(cols);
        std::vector<int> jpvt;
        std::vector<double> ht;
        geqp3(Asn, jpvt, ht);
        std::vector<double> diag(std::min(rows, cols));
        for (size_t i = 0; i < diag.size(); i++) diag[i] = Asn((int)i, (int)i);
        const int rank = choose_rank(diag, tol);
        rank_log.push_back({ilvl, self->order, rows, std::min(rank, rows)});
        if (rank >= rows) return;
        auto v = std::make_unique<Mat>(rows, rank);
        for (int j = 0; j < rank; j++)
            for (int i = 0; i < rows; i++) (*v)(i, j) = Asn(i, j);
        auto op = make_op(OP_ORTHOGONAL, self, nullptr, std::move(v));
        op->h.assign(ht.begin(), ht.begin() + rank);
        const Op* qop = op.get();
        push_op(std::move(op));
        Mat AsnP(rank, cols);
        for (int j = 0; j < cols; j++)
            for (int i = 0; i < rank && i <= j; i++) AsnP(i, jpvt[j]) = Asn(i, j);
        Cluster* sib = shrink_split(self, rank, &AsnP, *qop->A, qop->h, true);
        eliminate_cluster(sib);
    }
    // tree.cpp:1553-1608 (SPD / LLT): per level every cluster is scaled and sparsified in
    // list order, then the level merges; nothing is eliminated as an interior
    void factorize_lorasp() {
        if (!lorasp) throw std::runtime_error("factorize_lorasp() needs partition_lorasp()");
        if (symm != SPD || scale_kind != S_LLT || preserve)
            throw std::runtime_error("oracle: LoRaSp is restated for SPD / LLT without preservation");
        double t0 = now_s();
        for (ilvl = 0; ilvl < nlevels; ilvl++) {
            std::vector<Cluster*> cl;
            for (auto& s : bottom_current()) cl.push_back(s.get());
            for (auto s : cl) {
                scale_cluster(s);
                log[ilvl].rank_before.add(s->size);
                sparsify_farfield(s);
                log[ilvl].rank_after.add(s->size);
            }
            if (ilvl < nlevels - 1) merge_all();
            log[ilvl].dofs_left_spars = ndofs_left();
            log[ilvl].fact_nnz = nnz();
        }
        t_factorize = now_s() - t0;
    }
    void sparsify_cluster(Cluster* self) {  // tree.cpp:1417-1433
        if (!use_want_sparsify || self->sparsify) {
            log[ilvl].rank_before.add(self->size);
            if (preserve) {
                if (tol <= 1.0) sparsify_preserve_adaptive(self);
                else sparsify_preserve_only(self);
            } else {
                sparsify_adaptive_only(self);
            }
            log[ilvl].rank_after.add(self->size);
        } else {
            log[ilvl].ignored++;
        }
    }

    // ---- merge ------------------------------------------------------------------
    // tree.cpp:1106-1131
    void reset_size(Cluster* snew, std::map<Cluster*, int>& posparent) {
        int size = 0;
        for (auto sold : snew->children) { posparent[sold] = size; size += sold->size; }
        snew->reset_size(size);
        if (preserve) {  // tree.cpp:1115-1128
            snew->phi = std::make_unique<Mat>(size, nphi);
            int row = 0;
            for (auto sold : snew->children) {
                for (int j = 0; j < nphi; j++)
                    for (int i = 0; i < sold->size; i++) (*snew->phi)(row + i, j) = (*sold->phi)(i, j);
                row += sold->size;
            }
        }
        push_op(make_op(OP_MERGE, snew, nullptr, nullptr));
    }
    // tree.cpp:1133-1184
    void update_edges(Cluster* snew, std::map<Cluster*, int>& posparent) {
        std::map<int, std::pair<Cluster*, bool>> merged;  // keyed by order: iteration order only affects list order pre-sort
        for (auto sold : snew->children)
            for (auto& eold : sold->edgesOut) {
                Cluster* nnew = eold->n2->parent;
                auto it = merged.find(nnew->order);
                if (it == merged.end()) merged[nnew->order] = {nnew, eold->original};
                else if (!it->second.second) it->second.second = eold->original;
            }
        for (auto& kv : merged) {
            Cluster* nnew = kv.second.first;
            snew->add_edge(std::make_unique<Edge>(Edge{snew, nnew, std::make_unique<Mat>(nnew->size, snew->size), kv.second.second}));
        }
        snew->sort_edges();
        for (auto sold : snew->children) {
            for (auto& eold : sold->edgesOut) {
                Cluster* nold = eold->n2;
                Cluster* nnew = nold->parent;
                Edge* found = nullptr;
                for (auto& e : snew->edgesOut)
                    if (e->n2 == nnew) { found = e.get(); break; }
                int r0 = posparent[nold], c0 = posparent[sold];
                Mat& D = *found->A;
                Mat& S = *eold->A;
                for (int j = 0; j < S.c; j++)
                    for (int i = 0; i < S.r; i++) D(r0 + i, c0 + j) = S(i, j);
            }
            sold->edgesOut.clear();
            sold->edgesIn.clear();
        }
    }
    void merge_all() {  // tree.cpp:1435-1445
        current_bottom++;
        std::map<Cluster*, int> posparent;
        for (auto& s : bottom_current()) reset_size(s.get(), posparent);
        for (auto& s : bottom_current()) update_edges(s.get(), posparent);
    }

    // tree.cpp:1447-1551
    void factorize() {
        double t0 = now_s();
        if (preserve) {  // tree.cpp:1477-1485: phi_ = P^T phi split over the leaf clusters
            if (!symmetry()) throw std::runtime_error("oracle: preservation needs a symmetric matrix");
            const int n = N();
            if ((int)phi.size() != n * nphi || nphi <= 0) throw std::runtime_error("oracle: phi not set");
            for (auto& c : bottom_original()) {
                c->phi = std::make_unique<Mat>(c->size, nphi);
                for (int j = 0; j < nphi; j++)
                    for (int i = 0; i < c->size; i++) (*c->phi)(i, j) = phi[(size_t)perm[c->start + i] + (size_t)j * n];
            }
        }
        for (ilvl = 0; ilvl < nlevels; ilvl++) {
            double ta = now_s();
            {
                std::vector<Cluster*> elim;
                for (auto& s : bottom_current())
                    if (s->level == ilvl) elim.push_back(s.get());
                for (auto s : elim) eliminate_cluster(s);
                log[ilvl].dofs_left_elim = ndofs_left();
            }
            double tb = now_s();
            log[ilvl].t_elim = tb - ta;
            if (ilvl >= skip) {
                for (auto& s : bottom_current())
                    if (s->level > ilvl) scale_cluster(s.get());
                double tc = now_s();
                log[ilvl].t_scale = tc - tb;
                std::vector<Cluster*> sp;
                for (auto& s : bottom_current())
                    if (s->level > ilvl) sp.push_back(s.get());
                for (auto s : sp) sparsify_cluster(s);
                log[ilvl].t_spars = now_s() - tc;
            }
            double td = now_s();
            if (ilvl < nlevels - 1) merge_all();
            log[ilvl].t_merge = now_s() - td;
            log[ilvl].dofs_left_spars = ndofs_left();
            log[ilvl].fact_nnz = nnz();
        }
        t_factorize = now_s() - t0;
    }

    // tree.cpp:1610-1635
    void solve(double* xnat) {
        int n = N();
        std::vector<double> b(n);
        for (int i = 0; i < n; i++) b[i] = xnat[perm[i]];
        for (auto& c : bottom_original()) {
            if (c->children.empty()) std::copy(b.begin() + c->start, b.begin() + c->start + c->x.size(), c->x.begin());
            else std::fill(c->x.begin(), c->x.end(), 0.0);
        }
        for (auto& op : ops) op->fwd();
        for (auto& op : ops) op->diag();  // tree.cpp:1621-1624 (LDLT only)
        for (auto it = ops.rbegin(); it != ops.rend(); ++it) (*it)->bwd();
        for (auto& c : bottom_original())
            if (c->children.empty()) std::copy(c->x.begin(), c->x.end(), b.begin() + c->start);
        for (int i = 0; i < n; i++) xnat[perm[i]] = b[i];
    }

    // Current trailing matrix in permuted ordering as dense-coordinate triplets; tree.cpp:1730-1763
    void trailing(std::vector<int>& I, std::vector<int>& J, std::vector<double>& V) {
        for (auto& s : bottom_current()) {
            if (s->eliminated) continue;
            for (auto& e : s->edgesOut) {
                int n1 = e->n2->start, n2 = e->n2->size, s1 = s->start, s2 = s->size;
                for (int i_ = 0; i_ < n2; i_++)
                    for (int j_ = 0; j_ < s2; j_++) {
                        int i = n1 + i_, j = s1 + j_;
                        double v = (*e->A)(i_, j_);
                        if (symmetry() && i > j) { I.push_back(j); J.push_back(i); V.push_back(v); I.push_back(i); J.push_back(j); V.push_back(v); }
                        else if (symmetry() && i == j) { I.push_back(i); J.push_back(i); V.push_back(v); }
                        else if (!symmetry()) { I.push_back(i); J.push_back(j); V.push_back(v); }
                    }
            }
        }
    }
};

// y = A x (CSC, column traversal as in Eigen's sparse * dense)
static void spmv(const CSC& A, const double* x, double* y) {
    std::fill(y, y + A.n, 0.0);
    for (int j = 0; j < A.n; j++) {
        double xj = x[j];
        for (int k = A.colptr[j]; k < A.colptr[j + 1]; k++) y[A.rowval[k]] += A.val[k] * xj;
    }
}
static double dot(int n, const double* a, const double* b) {
    double s = 0;
    for (int i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

// Preconditioned CG; is.cpp:39-121.  Returns the iteration count (i+1).
static int cg(const CSC& A, const double* rhs, double* x, Tree& M, int iters, double tol, double* relres_out) {
    int n = A.n;
    std::vector<double> r(n), p(n), z(n), tmp(n);
    spmv(A, x, tmp.data());
    for (int i = 0; i < n; i++) r[i] = rhs[i] - tmp[i];
    double rhsNorm2 = dot(n, rhs, rhs);
    if (rhsNorm2 == 0) { std::fill(x, x + n, 0.0); return 0; }
    double threshold = tol * tol * rhsNorm2;
    double resNorm2 = dot(n, r.data(), r.data());
    if (relres_out) *relres_out = std::sqrt(resNorm2 / rhsNorm2);
    if (resNorm2 < threshold) return 0;
    p = r;
    M.solve(p.data());
    double absNew = dot(n, r.data(), p.data());
    int i = 0;
    while (i < iters) {
        spmv(A, p.data(), tmp.data());
        double alpha = absNew / dot(n, p.data(), tmp.data());
        for (int k = 0; k < n; k++) x[k] += alpha * p[k];
        for (int k = 0; k < n; k++) r[k] -= alpha * tmp[k];
        resNorm2 = dot(n, r.data(), r.data());
        if (resNorm2 < threshold) break;
        z = r;
        M.solve(z.data());
        double absOld = absNew;
        absNew = dot(n, r.data(), z.data());
        double beta = absNew / absOld;
        for (int k = 0; k < n; k++) p[k] = z[k] + beta * p[k];
        i++;
    }
    if (relres_out) *relres_out = std::sqrt(resNorm2 / rhsNorm2);
    return i + 1;
}

// Iterative refinement; is.cpp:12-37.
static int ir(const CSC& A, const double* rhs, double* x, Tree& M, int iters, double tol) {
    int n = A.n;
    std::vector<double> res(n), tmp(n);
    spmv(A, x, tmp.data());
    for (int k = 0; k < n; k++) res[k] = rhs[k] - tmp[k];
    double rhsNorm2 = dot(n, rhs, rhs);
    if (rhsNorm2 == 0) { std::fill(x, x + n, 0.0); return 0; }
    double threshold = tol * tol * rhsNorm2;
    double resNorm2 = dot(n, res.data(), res.data());
    int i = 1;
    while (resNorm2 >= threshold && i < iters) {
        M.solve(res.data());
        for (int k = 0; k < n; k++) x[k] += res[k];
        spmv(A, x, tmp.data());
        for (int k = 0; k < n; k++) res[k] = rhs[k] - tmp[k];
        resNorm2 = dot(n, res.data(), res.data());
        if (resNorm2 < threshold) break;
        i++;
    }
    return i;
}

// ---------------------------------------------------------------------------------
// Restarted GMRES with Householder Arnoldi, left preconditioned; is.cpp:123-300.  The
// reference is Eigen's GMRES (unsupported/Eigen/src/IterativeSolvers/GMRES.h, Eigen
// 3.3.x) with the preconditioner's solve in place of Eigen's preconditioner: the
// Householder helpers below restate Eigen's published makeHouseholder /
// applyHouseholderOnTheLeft and the real makeGivens / applyOnTheLeft of JacobiRotation.
// ---------------------------------------------------------------------------------
namespace gm {
// x (length len) = beta e_0 after I - tau [1; ess][1; ess]^T; ess has len - 1 entries
static void make_householder(const double* x, int len, double* ess, double& tau, double& beta) {
    double tail = 0;
    for (int i = 1; i < len; i++) tail += x[i] * x[i];
    const double c0 = x[0];
    if (tail <= std::numeric_limits<double>::min()) {
        tau = 0;
        beta = c0;
        for (int i = 1; i < len; i++) ess[i - 1] = 0;
        return;
    }
    beta = std::sqrt(c0 * c0 + tail);
    if (c0 >= 0) beta = -beta;
    for (int i = 1; i < len; i++) ess[i - 1] = x[i] / (c0 - beta);
    tau = (beta - c0) / beta;
}
// y (length len) <- (I - tau [1; ess][1; ess]^T) y
static void apply_householder(double* y, int len, const double* ess, double tau) {
    if (len == 1) {
        y[0] *= 1.0 - tau;
        return;
    }
    if (tau == 0) return;
    double t = y[0];
    for (int i = 1; i < len; i++) t += ess[i - 1] * y[i];
    y[0] -= tau * t;
    for (int i = 1; i < len; i++) y[i] -= tau * ess[i - 1] * t;
}
struct Givens {
    double c = 1, s = 0;
};
// G such that G^T applied to (p, q) gives (r, 0)
static Givens make_givens(double p, double q) {
    Givens g;
    if (q == 0) {
        g.c = p < 0 ? -1 : 1;
        g.s = 0;
    } else if (p == 0) {
        g.c = 0;
        g.s = q < 0 ? 1 : -1;
    } else if (std::fabs(p) > std::fabs(q)) {
        double t = q / p, u = std::sqrt(1 + t * t);
        if (p < 0) u = -u;
        g.c = 1 / u;
        g.s = -t * g.c;
    } else {
        double t = p / q, u = std::sqrt(1 + t * t);
        if (q < 0) u = -u;
        g.s = -1 / u;
        g.c = -t * g.s;
    }
    return g;
}
// rows (i, j) of v <- G^T (rows i, j): x' = c x - s y, y' = s x + c y
static void apply_givens_t(double* v, int i, int j, const Givens& g) {
    const double x = v[i], y = v[j];
    v[i] = g.c * x - g.s * y;
    v[j] = g.s * x + g.c * y;
}
}  // namespace gm

static int gmres(const CSC& A, const double* rhs, double* x, Tree& M, int iters, int restart, double tol,
                 double* relres_out) {
    const int m = A.n;
    if (std::sqrt(dot(m, rhs, rhs)) <= std::numeric_limits<double>::min()) {
        std::fill(x, x + m, 0.0);
        if (relres_out) *relres_out = 0;
        return 1;
    }
    int it = 0;
    std::vector<double> r0(m), t(m), v(m);
    // H: reflector i in column i (its essential part at rows i+1..m-1); above the diagonal,
    // the upper triangle of the rotated Hessenberg matrix
    std::vector<double> H((size_t)m * (restart + 1), 0.0), w(restart + 1, 0.0), tau(restart + 1, 0.0);
    std::vector<gm::Givens> G(restart);
    auto col = [&](int i) { return H.data() + (size_t)i * m; };
    // the stopping test divides by the norm of the FIRST preconditioned residual, also
    // after a restart (r0Norm is computed once, is.cpp:161)
    double r0norm = -1;
    auto start = [&]() {  // preconditioned residual and the first reflector
        spmv(A, x, t.data());
        for (int i = 0; i < m; i++) r0[i] = rhs[i] - t[i];
        M.solve(r0.data());
        if (r0norm < 0) r0norm = std::sqrt(dot(m, r0.data(), r0.data()));
        std::fill(H.begin(), H.end(), 0.0);
        std::fill(w.begin(), w.end(), 0.0);
        std::fill(tau.begin(), tau.end(), 0.0);
        double beta;
        gm::make_householder(r0.data(), m, col(0) + 1, tau[0], beta);
        w[0] = beta;
    };
    start();
    if (r0norm == 0) {
        if (relres_out) *relres_out = 0;
        return 1;
    }
    double err = 1.0;
    for (int k = 1; k <= restart; ++k) {
        ++it;
        std::fill(v.begin(), v.end(), 0.0);
        v[k - 1] = 1.0;
        for (int i = k - 1; i >= 0; --i) gm::apply_householder(v.data() + i, m - i, col(i) + i + 1, tau[i]);
        spmv(A, v.data(), t.data());
        v = t;
        M.solve(v.data());
        for (int i = 0; i < k; ++i) gm::apply_householder(v.data() + i, m - i, col(i) + i + 1, tau[i]);
        double tailsq = 0;
        for (int i = k; i < m; i++) tailsq += v[i] * v[i];
        if (tailsq != 0.0 && k < m) {
            double beta;
            gm::make_householder(v.data() + k, m - k, col(k) + k + 1, tau[k], beta);
            gm::apply_householder(v.data() + k, m - k, col(k) + k + 1, tau[k]);
        }
        for (int i = 0; i + 1 < k; ++i) gm::apply_givens_t(v.data(), i, i + 1, G[i]);
        if (k < m && v[k] != 0.0) {
            G[k - 1] = gm::make_givens(v[k - 1], v[k]);
            gm::apply_givens_t(v.data(), k - 1, k, G[k - 1]);
            gm::apply_givens_t(w.data(), k - 1, k, G[k - 1]);
        }
        for (int i = 0; i < k; i++) col(k - 1)[i] = v[i];
        err = std::fabs(w[k]) / r0norm;
        const bool stop = (k == m || err < tol || it == iters);
        if (stop || k == restart) {
            // y = R^{-1} w[0:k] (R: upper triangle of H), then x += H_0 ... H_{k-1} [y; 0]
            std::vector<double> y(w.begin(), w.begin() + k), xn(m, 0.0);
            for (int i = k - 1; i >= 0; i--) {
                double s = y[i];
                for (int j = i + 1; j < k; j++) s -= col(j)[i] * y[j];
                y[i] = s / col(i)[i];
            }
            for (int i = k - 1; i >= 0; --i) {
                xn[i] += y[i];
                gm::apply_householder(xn.data() + i, m - i, col(i) + i + 1, tau[i]);
            }
            for (int i = 0; i < m; i++) x[i] += xn[i];
            if (stop) break;
            k = 0;
            start();
        }
    }
    if (relres_out) *relres_out = err;
    return it;
}

}  // namespace orc

// =================================================================================
// C API (ctypes), oracle only
// =================================================================================
using namespace orc;

struct OrcHandle {
    std::unique_ptr<Tree> t;
    CSC A;
    std::vector<double> X;
    std::string err;
};

static CSC make_csc(int n, const int* colptr, const int* rowval, const double* val) {
    CSC A;
    A.n = n;
    A.colptr.assign(colptr, colptr + n + 1);
    int nnz = colptr[n];
    A.rowval.assign(rowval, rowval + nnz);
    if (val) A.val.assign(val, val + nnz);
    else A.val.assign(nnz, 1.0);
    return A;
}

extern "C" {

void* orc_create(int nlevels) {
    auto h = new OrcHandle();
    h->t = std::make_unique<Tree>(nlevels);
    return h;
}
void orc_destroy(void* p) { delete (OrcHandle*)p; }
const char* orc_error(void* p) { return ((OrcHandle*)p)->err.c_str(); }
void orc_set_tol(void* p, double tol) { ((OrcHandle*)p)->t->tol = tol; }
void orc_set_skip(void* p, int skip) { ((OrcHandle*)p)->t->skip = skip; }
void orc_set_symm_kind(void* p, int k) { ((OrcHandle*)p)->t->symm = k; }
void orc_set_scaling_kind(void* p, int k) { ((OrcHandle*)p)->t->scale_kind = k; }
void orc_set_use_sparsify(void* p, int u) { ((OrcHandle*)p)->t->use_want_sparsify = u != 0; }
// Load CBLAS / LAPACKE entry points from a shared library (names with the given prefix,
// e.g. "scipy_" for scipy's bundled OpenBLAS) and route the dense kernels through them;
// threads > 0 sets the library's thread count when it exports <prefix>openblas_set_num_threads.
// path == nullptr: back to the restated kernels.  Returns 0, or -1 when a symbol is missing.
int orc_use_lapack(const char* path, const char* prefix, int threads) {
    if (!path) {
        lapk::gemm = nullptr;
        lapk::syrk = nullptr;
        lapk::trsm = nullptr;
        lapk::potrf = nullptr;
        lapk::geqp3 = nullptr;
        return 0;
    }
    void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
    if (!h) return -1;
    const std::string pre = prefix ? prefix : "";
    auto sym = [&](const char* name) { return dlsym(h, (pre + name).c_str()); };
    auto g = (lapk::gemm_t)sym("cblas_dgemm");
    auto s = (lapk::syrk_t)sym("cblas_dsyrk");
    auto t = (lapk::trsm_t)sym("cblas_dtrsm");
    auto p = (lapk::potrf_t)sym("LAPACKE_dpotrf");
    auto q = (lapk::geqp3_t)sym("LAPACKE_dgeqp3");
    if (!g || !s || !t || !p || !q) return -1;
    if (threads > 0) {
        auto nt = (lapk::threads_t)sym("openblas_set_num_threads");
        if (nt) nt(threads);
    }
    lapk::gemm = g;
    lapk::syrk = s;
    lapk::trsm = t;
    lapk::potrf = p;
    lapk::geqp3 = q;
    return 0;
}
void orc_set_preserve(void* p, int on) { ((OrcHandle*)p)->t->preserve = on != 0; }
// phi: n x nphi, column-major, natural ordering (copied)
void orc_set_phi(void* p, const double* phi, int n, int nphi) {
    auto t = ((OrcHandle*)p)->t.get();
    t->phi.assign(phi, phi + (size_t)n * nphi);
    t->nphi = nphi;
}
void orc_set_Xcoo(void* p, const double* X, int dim, int n) {
    auto h = (OrcHandle*)p;
    h->X.assign(X, X + (size_t)dim * n);
    h->t->X = h->X.data();
    h->t->dim = dim;
    h->t->geo = true;
}

int orc_partition(void* p, int n, const int* colptr, const int* rowval) {
    auto h = (OrcHandle*)p;
    try {
        h->t->partition(make_csc(n, colptr, rowval, nullptr));
    } catch (std::exception& e) { h->err = e.what(); return -1; }
    return 0;
}
// out: 6*N ints: self.lvl self.sep l.lvl l.sep r.lvl r.sep per dof (natural ordering)
void orc_get_partition(void* p, int* out) {
    auto& part = ((OrcHandle*)p)->t->part;
    for (size_t i = 0; i < part.size(); i++) {
        out[6 * i + 0] = part[i].self.lvl; out[6 * i + 1] = part[i].self.sep;
        out[6 * i + 2] = part[i].l.lvl;    out[6 * i + 3] = part[i].l.sep;
        out[6 * i + 4] = part[i].r.lvl;    out[6 * i + 5] = part[i].r.sep;
    }
}
void orc_get_perm(void* p, int* perm) {
    auto& v = ((OrcHandle*)p)->t->perm;
    std::copy(v.begin(), v.end(), perm);
}
int orc_num_clusters(void* p, int lvl) { return (int)((OrcHandle*)p)->t->bottoms[lvl].size(); }
// per cluster at hierarchy level lvl: start size level order sparsify parent_order
void orc_get_clusters(void* p, int lvl, int* out) {
    int k = 0;
    for (auto& c : ((OrcHandle*)p)->t->bottoms[lvl]) {
        out[6 * k + 0] = c->start; out[6 * k + 1] = c->size; out[6 * k + 2] = c->level;
        out[6 * k + 3] = c->order; out[6 * k + 4] = c->sparsify; out[6 * k + 5] = c->parent ? c->parent->order : -1;
        k++;
    }
}
int orc_assemble(void* p, int n, const int* colptr, const int* rowval, const double* val) {
    auto h = (OrcHandle*)p;
    try {
        h->A = make_csc(n, colptr, rowval, val);
        h->t->assemble(h->A);
    } catch (std::exception& e) { h->err = e.what(); return -1; }
    return 0;
}
// trailing matrix triplets; returns count, fills when buffers non-null
int orc_trailing(void* p, int* I, int* J, double* V) {
    std::vector<int> i, j;
    std::vector<double> v;
    ((OrcHandle*)p)->t->trailing(i, j, v);
    if (I) { std::copy(i.begin(), i.end(), I); std::copy(j.begin(), j.end(), J); std::copy(v.begin(), v.end(), V); }
    return (int)i.size();
}
int orc_partition_lorasp(void* p, int n, const int* colptr, const int* rowval) {
    auto h = (OrcHandle*)p;
    try {
        h->t->partition_lorasp(make_csc(n, colptr, rowval, nullptr));
    } catch (std::exception& e) { h->err = e.what(); return -1; }
    return 0;
}
void orc_get_rb_parts(void* p, int* out) {
    auto& r = ((OrcHandle*)p)->t->rb_parts;
    std::copy(r.begin(), r.end(), out);
}
int orc_factorize_lorasp(void* p) {
    auto h = (OrcHandle*)p;
    try {
        h->t->factorize_lorasp();
    } catch (std::exception& e) { h->err = e.what(); return -1; }
    return 0;
}
int orc_factorize(void* p) {
    auto h = (OrcHandle*)p;
    try {
        h->t->factorize();
    } catch (std::exception& e) { h->err = e.what(); return -1; }
    return 0;
}
void orc_solve(void* p, double* x) { ((OrcHandle*)p)->t->solve(x); }
void orc_solve_multi(void* p, double* x, int nrhs, int ld) {
    for (int k = 0; k < nrhs; k++) ((OrcHandle*)p)->t->solve(x + (size_t)k * ld);
}
int orc_cg(void* p, const double* b, double* x, int iters, double tol, double* relres) {
    auto h = (OrcHandle*)p;
    return cg(h->A, b, x, *h->t, iters, tol, relres);
}
int orc_gmres(void* p, const double* b, double* x, int iters, int restart, double tol, double* relres) {
    auto h = (OrcHandle*)p;
    return gmres(h->A, b, x, *h->t, iters, restart, tol, relres);
}
int orc_ir(void* p, const double* b, double* x, int iters, double tol) {
    auto h = (OrcHandle*)p;
    return ir(h->A, b, x, *h->t, iters, tol);
}
long long orc_nnz(void* p) { return ((OrcHandle*)p)->t->nnz(); }
int orc_get_stop(void* p) { return ((OrcHandle*)p)->t->get_stop(); }
// per level: dofs_nd dofs_left_nd dofs_left_elim dofs_left_spars rank_before_sum rank_after_sum
//            rank_after_count ignored nbrs_sum nbrs_count
void orc_get_log(void* p, long long* out) {
    auto& L = ((OrcHandle*)p)->t->log;
    for (size_t l = 0; l < L.size(); l++) {
        long long* o = out + 11 * l;
        o[0] = L[l].dofs_nd; o[1] = L[l].dofs_left_nd; o[2] = L[l].dofs_left_elim; o[3] = L[l].dofs_left_spars;
        o[4] = L[l].rank_before.sum; o[5] = L[l].rank_after.sum; o[6] = L[l].rank_after.count; o[7] = L[l].ignored;
        o[8] = L[l].nbrs.sum; o[9] = L[l].nbrs.count; o[10] = L[l].fact_nnz;
    }
}
// per level: t_elim t_scale t_spars t_merge flops_potf flops_trsm flops_gemm flops_geqp3
void orc_get_prof(void* p, double* out) {
    auto& L = ((OrcHandle*)p)->t->log;
    for (size_t l = 0; l < L.size(); l++) {
        double* o = out + 8 * l;
        o[0] = L[l].t_elim; o[1] = L[l].t_scale; o[2] = L[l].t_spars; o[3] = L[l].t_merge;
        o[4] = L[l].flops_potf; o[5] = L[l].flops_trsm; o[6] = L[l].flops_gemm; o[7] = L[l].flops_geqp3;
    }
}
void orc_get_times(void* p, double* out) {
    auto t = ((OrcHandle*)p)->t.get();
    out[0] = t->t_partition; out[1] = t->t_assemble; out[2] = t->t_factorize;
}
int orc_num_ranks(void* p) { return (int)((OrcHandle*)p)->t->rank_log.size(); }
void orc_get_ranks(void* p, int* out) {
    auto& r = ((OrcHandle*)p)->t->rank_log;
    for (size_t i = 0; i < r.size(); i++)
        for (int k = 0; k < 4; k++) out[4 * i + k] = r[i][k];
}
// Op list introspection: per op kind, level, self order, nbr order, ns, nn, rows(A), cols(A)
int orc_num_ops(void* p) { return (int)((OrcHandle*)p)->t->ops.size(); }
void orc_get_ops(void* p, int* out) {
    int k = 0;
    for (auto& op : ((OrcHandle*)p)->t->ops) {
        int* o = out + 8 * k;
        o[0] = op->kind; o[1] = op->ilvl; o[2] = op->self ? op->self->order : -1; o[3] = op->nbr ? op->nbr->order : -1;
        o[4] = op->ns; o[5] = op->nn; o[6] = op->A ? op->A->r : 0; o[7] = op->A ? op->A->c : 0;
        k++;
    }
}
// Copy the A matrix of op #idx (column-major) into out; returns number of entries
long long orc_get_op_matrix(void* p, int idx, double* out) {
    auto it = ((OrcHandle*)p)->t->ops.begin();
    std::advance(it, idx);
    if (!(*it)->A) return 0;
    auto& v = (*it)->A->v;
    if (out) std::copy(v.begin(), v.end(), out);
    return (long long)v.size();
}
// U factor (n x n, column-major) and row permutation of a PLUQ op
long long orc_get_op_u(void* p, int idx, double* out) {
    auto it = ((OrcHandle*)p)->t->ops.begin();
    std::advance(it, idx);
    if (!(*it)->U) return 0;
    auto& v = (*it)->U->v;
    if (out) std::copy(v.begin(), v.end(), out);
    return (long long)v.size();
}
// sign(D) of a ScalingLDLT op (also carried by the Gemm ops of an LDLT pivot)
int orc_get_op_signs(void* p, int idx, double* out) {
    auto it = ((OrcHandle*)p)->t->ops.begin();
    std::advance(it, idx);
    auto& s = (*it)->s;
    if (out) std::copy(s.begin(), s.end(), out);
    return (int)s.size();
}
int orc_get_op_perm(void* p, int idx, int* out) {
    auto it = ((OrcHandle*)p)->t->ops.begin();
    std::advance(it, idx);
    auto& q = (*it)->p;
    if (out) std::copy(q.begin(), q.end(), out);
    return (int)q.size();
}
int orc_get_op_tau(void* p, int idx, double* out) {
    auto it = ((OrcHandle*)p)->t->ops.begin();
    std::advance(it, idx);
    auto& h = (*it)->h;
    if (out) std::copy(h.begin(), h.end(), out);
    return (int)h.size();
}

// Dense kernels exposed for cross-checks against LAPACK
int orc_dense_potf(int n, double* A) {
    Mat M(n, n);
    std::copy(A, A + (size_t)n * n, M.v.begin());
    int info = potf(M);
    std::copy(M.v.begin(), M.v.end(), A);
    return info;
}
void orc_dense_geqp3(int m, int n, double* A, int* jpvt, double* tau) {
    Mat M(m, n);
    std::copy(A, A + (size_t)m * n, M.v.begin());
    std::vector<int> jp;
    std::vector<double> t;
    geqp3(M, jp, t);
    std::copy(M.v.begin(), M.v.end(), A);
    std::copy(jp.begin(), jp.end(), jpvt);
    std::copy(t.begin(), t.end(), tau);
}
int orc_dense_getf(int n, double* A, int* perm) {
    Mat M(n, n);
    std::copy(A, A + (size_t)n * n, M.v.begin());
    std::vector<int> p;
    int info = getf(M, p);
    std::copy(M.v.begin(), M.v.end(), A);
    if (info == 0) std::copy(p.begin(), p.end(), perm);
    return info;
}
int orc_choose_rank(const double* s, int n, double tol) {
    return choose_rank(std::vector<double>(s, s + n), tol);
}
void orc_spmv(void* p, const double* x, double* y) { spmv(((OrcHandle*)p)->A, x, y); }

}  // extern "C"

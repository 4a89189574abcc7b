// The reference command-line driver's flow (tests/spaND.cpp:208-367 of spaND_public)
// compiled against the C++ drop-in spaND::Tree (spand_public_gb300/csrc/tree.h) and linked
// with libspand_gb300.so: setters, partition, assemble, factorize inside try/catch,
// print_log, the get_stop / nnz queries, one solve of a random right-hand side and CG.
//
//   cli_flow <grid side> <dimension 2|3> <levels> <tol> [fp32 0|1]
//
// Prints "<<<<key=value" lines like the reference driver and exits non-zero when the CG
// does not reach 1e-10 or an unexpected exception escapes.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <random>
#include <string>
#include <vector>

#include "tree.h"

// -Laplacian with the 2d+1-point stencil on an n^d grid (row-major grid index, Dirichlet),
// as mats/neglapl_*.mm; CSC with sorted rows.
static spand::Csc neglapl(int n, int d) {
    const int N = d == 2 ? n * n : n * n * n;
    spand::Csc A;
    A.n = N;
    A.colptr.push_back(0);
    for (int j = 0; j < N; j++) {
        int c[3] = {0, 0, 0};
        int r = j;
        for (int k = d - 1; k >= 0; k--) {
            c[k] = r % n;
            r /= n;
        }
        std::vector<int> rows;
        int stride = 1;
        for (int k = d - 1; k >= 0; k--) {
            if (c[k] > 0) rows.push_back(j - stride);
            if (c[k] < n - 1) rows.push_back(j + stride);
            stride *= n;
        }
        rows.push_back(j);
        std::sort(rows.begin(), rows.end());
        for (int i : rows) {
            A.rowval.push_back(i);
            A.val.push_back(i == j ? 2.0 * d : -1.0);
        }
        A.colptr.push_back((int)A.rowval.size());
    }
    return A;
}

// dim x N coordinates, first coordinate the slowest grid index (linspace_nd, src/util.cpp:488-517)
static std::vector<double> coords(int n, int d) {
    const int N = d == 2 ? n * n : n * n * n;
    std::vector<double> X((size_t)d * N);
    for (int j = 0; j < N; j++) {
        int r = j;
        for (int k = d - 1; k >= 0; k--) {
            X[(size_t)j * d + k] = r % n;
            r /= n;
        }
    }
    return X;
}

static void spmv(const spand::Csc& A, const std::vector<double>& x, std::vector<double>& y) {
    y.assign(A.n, 0.0);
    for (int j = 0; j < A.n; j++)
        for (int k = A.colptr[j]; k < A.colptr[j + 1]; k++) y[A.rowval[k]] += A.val[k] * x[j];
}

static double norm(const std::vector<double>& v) {
    double s = 0;
    for (double e : v) s += e * e;
    return std::sqrt(s);
}

int main(int argc, char** argv) {
    if (argc < 5) {
        fprintf(stderr, "usage: %s n dim levels tol [fp32]\n", argv[0]);
        return 2;
    }
    const int n = atoi(argv[1]), dim = atoi(argv[2]), nlevels = atoi(argv[3]);
    const double tol = atof(argv[4]);
    const bool fp32 = argc > 5 && atoi(argv[5]) != 0;
    spand::Csc A = neglapl(n, dim);
    std::vector<double> X = coords(n, dim);
    const int N = A.n;
    try {
        spaND::Tree t(nlevels);
        t.set_verb(true);
        t.set_symm_kind(spaND::SymmKind::SPD);
        t.set_tol(tol);
        t.set_skip(0);
        t.set_preserve(false);
        t.set_use_geo(true);
        t.set_Xcoo(X.data(), dim, N);
        t.set_scaling_kind(spaND::ScalingKind::LLT);
        t.set_part_kind(spaND::PartKind::MND);
        t.set_use_sparsify(true);
        t.set_fp32(fp32);
        printf("<<<<N=%d\n<<<<nlevels=%d\n<<<<tol=%g\n", N, nlevels, tol);
        t.partition(A);
        t.assemble(A);
        try {
            t.factorize();
        } catch (std::exception& ex) {
            printf("%s", ex.what());
            printf("<<<<FAILED\n");
            return 1;
        }
        t.print_log();
        printf("<<<<tpart=%g\n<<<<tassm=%g\n<<<<tfact=%g\n", t.t_partition, t.t_assemble, t.t_factorize);
        printf("<<<<stop=%d\n<<<<nnzfact=%lld\n", t.get_stop(), t.nnz());
        // one solve of a random right-hand side (U(-1, 1), seed 2019)
        std::mt19937 gen(2019);
        std::uniform_real_distribution<double> U(-1.0, 1.0);
        std::vector<double> b(N), x, Ax;
        for (double& e : b) e = U(gen);
        x = b;
        t.solve(x.data());
        spmv(A, x, Ax);
        for (int i = 0; i < N; i++) Ax[i] -= b[i];
        const double one_shot = norm(Ax) / norm(b);
        printf("One-time solve (Random b):\n<<<<|Ax-b|/|b| : %g\n", one_shot);
        // CG from zero
        std::vector<double> xc(N, 0.0);
        const int iter = spaND::cg(A, b.data(), xc.data(), t, 100, 1e-10, true);
        spmv(A, xc, Ax);
        for (int i = 0; i < N; i++) Ax[i] -= b[i];
        const double res = norm(Ax) / norm(b);
        printf("CG: #iterations: %d, residual |Ax-b|/|b|: %g\n<<<<CG=%d\n", iter, res, iter);
        if (!(one_shot < 1.0) || !(res < 1e-9)) {
            printf("<<<<BAD\n");
            return 1;
        }
        // a non-SPD matrix raises the reference's message from factorize()
        spand::Csc B = A;
        for (double& v : B.val) v = -v;
        spaND::Tree t2(nlevels);
        t2.set_verb(false);
        t2.set_tol(tol);
        t2.set_use_geo(true);
        t2.set_Xcoo(X.data(), dim, N);
        t2.partition(B);
        t2.assemble(B);
        bool threw = false;
        try {
            t2.factorize();
        } catch (std::runtime_error& ex) {
            threw = std::string(ex.what()).find("Non-SPD Pivot") != std::string::npos;
        }
        printf("<<<<nonspd_throws=%d\n", threw ? 1 : 0);
        if (!threw) return 1;
    } catch (std::exception& ex) {
        printf("unexpected exception: %s\n", ex.what());
        return 1;
    } catch (spand::DeviceError& ex) {
        printf("unexpected device error: %s\n", ex.msg.c_str());
        return 1;
    }
    printf("<<<<OK\n");
    return 0;
}

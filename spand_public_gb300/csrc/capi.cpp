// extern "C" boundary (include/spand_gb300.h) over spaND::Tree.
#include <algorithm>
#include <cstring>
#include <exception>
#include <string>

#include "../../include/spand_gb300.h"
#include "forest.h"
#include "tree.h"

struct spand_tree {
    spaND::Tree* t;
    int geo = 0;
};

struct spand_forest {
    spaND::Forest* f;
};

static thread_local std::string g_err;

static int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

template <typename F>
static int guard(F&& f) {
    try {
        f();
        g_err.clear();
        return SPAND_OK;
    } catch (std::invalid_argument& e) {
        return fail(SPAND_ERR_ARG, e.what());
    } catch (std::logic_error& e) {
        return fail(SPAND_ERR_STATE, e.what());
    } catch (std::runtime_error& e) {
        std::string m = e.what();
        if (m.find("Non-SPD") != std::string::npos || m.find("Singular Pivot") != std::string::npos)
            return fail(SPAND_ERR_NOT_SPD, m);
        if (m.find("cuda") != std::string::npos || m.find("CUDA") != std::string::npos) return fail(SPAND_ERR_CUDA, m);
        return fail(SPAND_ERR_UNSUPPORTED, m);
    } catch (spand::DeviceError& e) {
        return fail(e.status, e.msg);
    } catch (std::exception& e) {
        return fail(SPAND_ERR_CUDA, e.what());
    }
}

static spand::Csc make_csc(int n, const int* colptr, const int* rowval, const double* vals) {
    if (n < 0 || !colptr || (!rowval && colptr[n] > 0)) throw std::invalid_argument("invalid CSC arrays");
    spand::Csc A;
    A.n = n;
    A.colptr.assign(colptr, colptr + n + 1);
    const int nnz = colptr[n];
    A.rowval.assign(rowval, rowval + nnz);
    if (vals) A.val.assign(vals, vals + nnz);
    else A.val.assign(nnz, 1.0);
    for (int j = 0; j < n; j++) {
        if (colptr[j + 1] < colptr[j]) throw std::invalid_argument("colptr must be non-decreasing");
        for (int k = colptr[j]; k < colptr[j + 1]; k++) {
            if (rowval[k] < 0 || rowval[k] >= n) throw std::invalid_argument("row index out of range");
            if (k > colptr[j] && rowval[k] <= rowval[k - 1]) throw std::invalid_argument("row indices must be sorted and unique");
        }
    }
    return A;
}

#define CHECK_T(t) \
    if (!(t) || !(t)->t) return fail(SPAND_ERR_ARG, "null tree")

extern "C" {

const char* spand_last_error(void) { return g_err.c_str(); }

int spand_tree_create(spand_tree** out, int nlevels) {
    if (!out) return fail(SPAND_ERR_ARG, "null output pointer");
    return guard([&] {
        auto* h = new spand_tree();
        h->t = new spaND::Tree(nlevels);
        *out = h;
    });
}

int spand_tree_destroy(spand_tree* t) {
    if (!t) return SPAND_OK;
    return guard([&] {
        delete t->t;
        delete t;
    });
}

int spand_tree_set_verb(spand_tree* t, int v) { CHECK_T(t); t->t->set_verb(v != 0); return SPAND_OK; }
int spand_tree_set_use_geo(spand_tree* t, int g) { CHECK_T(t); t->t->set_use_geo(g != 0); return SPAND_OK; }
int spand_tree_set_Xcoo(spand_tree* t, const double* X, int dim, int n) {
    CHECK_T(t);
    if (!X || dim <= 0 || n < 0) return fail(SPAND_ERR_ARG, "invalid coordinates");
    return guard([&] { t->t->set_Xcoo(X, dim, n); });
}
int spand_tree_set_tol(spand_tree* t, double tol) { CHECK_T(t); t->t->set_tol(tol); return SPAND_OK; }
int spand_tree_set_skip(spand_tree* t, int skip) { CHECK_T(t); t->t->set_skip(skip); return SPAND_OK; }
int spand_tree_set_scaling_kind(spand_tree* t, int k) {
    CHECK_T(t);
    if (k < 0 || k > 5) return fail(SPAND_ERR_ARG, "unknown scaling kind");
    t->t->set_scaling_kind((spaND::ScalingKind)k);
    return SPAND_OK;
}
int spand_tree_set_symm_kind(spand_tree* t, int k) {
    CHECK_T(t);
    if (k < 0 || k > 2) return fail(SPAND_ERR_ARG, "unknown symmetry kind");
    t->t->set_symm_kind((spaND::SymmKind)k);
    return SPAND_OK;
}
int spand_tree_set_part_kind(spand_tree* t, int k) {
    CHECK_T(t);
    if (k < 0 || k > 1) return fail(SPAND_ERR_ARG, "unknown partition kind");
    t->t->set_part_kind((spaND::PartKind)k);
    return SPAND_OK;
}
int spand_tree_set_use_sparsify(spand_tree* t, int u) { CHECK_T(t); t->t->set_use_sparsify(u != 0); return SPAND_OK; }
int spand_tree_set_fp32(spand_tree* t, int f) { CHECK_T(t); t->t->set_fp32(f != 0); return SPAND_OK; }
int spand_tree_set_preserve(spand_tree* t, int p) { CHECK_T(t); t->t->set_preserve(p != 0); return SPAND_OK; }
int spand_tree_set_phi(spand_tree* t, const double* phi, int n, int nphi) {
    CHECK_T(t);
    return guard([&] { t->t->set_phi(phi, n, nphi); });
}

int spand_tree_partition(spand_tree* t, int n, const int* colptr, const int* rowval, int* sepids) {
    CHECK_T(t);
    return guard([&] {
        auto part = t->t->partition(make_csc(n, colptr, rowval, nullptr));
        if (sepids)
            for (int i = 0; i < n; i++) {
                sepids[6 * i + 0] = part[i].self.lvl; sepids[6 * i + 1] = part[i].self.sep;
                sepids[6 * i + 2] = part[i].l.lvl;    sepids[6 * i + 3] = part[i].l.sep;
                sepids[6 * i + 4] = part[i].r.lvl;    sepids[6 * i + 5] = part[i].r.sep;
            }
    });
}

int spand_tree_partition_lorasp(spand_tree* t, int n, const int* colptr, const int* rowval, int* parts) {
    CHECK_T(t);
    return guard([&] {
        auto p = t->t->partition_lorasp(make_csc(n, colptr, rowval, nullptr));
        if (parts) std::copy(p.begin(), p.end(), parts);
    });
}

int spand_tree_assemble(spand_tree* t, int n, const int* colptr, const int* rowval, const double* vals) {
    CHECK_T(t);
    if (!vals) return fail(SPAND_ERR_ARG, "null values");
    return guard([&] {
        if (!t->t->assemble_same_pattern(n, colptr, rowval, vals)) t->t->assemble(make_csc(n, colptr, rowval, vals));
    });
}

int spand_tree_factorize(spand_tree* t) {
    CHECK_T(t);
    return guard([&] { t->t->factorize(); });
}

int spand_tree_factorize_lorasp(spand_tree* t) {
    CHECK_T(t);
    return guard([&] { t->t->factorize_lorasp(); });
}

int spand_tree_solve(spand_tree* t, double* x, int nrhs, int ld) {
    CHECK_T(t);
    if (!x || nrhs < 1 || ld < t->t->get_N()) return fail(SPAND_ERR_ARG, "invalid vector arguments");
    return guard([&] { t->t->solve(x, nrhs, ld); });
}

int spand_tree_solve_device(spand_tree* t, double* x, int nrhs, int ld) {
    CHECK_T(t);
    if (!x || nrhs < 1 || ld < t->t->get_N()) return fail(SPAND_ERR_ARG, "invalid vector arguments");
    return guard([&] { t->t->solve_device(x, nrhs, ld); });
}

int spand_tree_solve_device_noalloc(spand_tree* t, double* x, int nrhs, int ld) {
    CHECK_T(t);
    if (!x || nrhs < 1 || ld < t->t->get_N()) return fail(SPAND_ERR_ARG, "invalid vector arguments");
    return guard([&] { t->t->solve_device_noalloc(x, nrhs, ld); });
}

int spand_cg(spand_tree* t, const double* b, double* x, int iters, double tol, int verb, int* iters_out,
             double* relres_out) {
    CHECK_T(t);
    if (!b || !x) return fail(SPAND_ERR_ARG, "null vector");
    return guard([&] {
        double rr = 0;
        int it = spaND::cg(t->t->matrix(), b, x, *t->t, iters, tol, verb != 0, &rr);
        if (iters_out) *iters_out = it;
        if (relres_out) *relres_out = rr;
    });
}

int spand_gmres(spand_tree* t, const double* b, double* x, int iters, int restart, double tol, int verb,
                int* iters_out, double* relres_out) {
    CHECK_T(t);
    if (!b || !x) return fail(SPAND_ERR_ARG, "null vector");
    if (restart < 1) return fail(SPAND_ERR_ARG, "restart < 1");
    return guard([&] {
        double rr = 0;
        int it = spaND::gmres(t->t->matrix(), b, x, *t->t, iters, restart, tol, verb != 0, &rr);
        if (iters_out) *iters_out = it;
        if (relres_out) *relres_out = rr;
    });
}

int spand_gmres_device(spand_tree* t, const double* b, double* x, int iters, int restart, double tol,
                       int* iters_out, double* relres_out) {
    CHECK_T(t);
    if (!b || !x) return fail(SPAND_ERR_ARG, "null vector");
    if (restart < 1) return fail(SPAND_ERR_ARG, "restart < 1");
    return guard([&] {
        if (!t->t->device()) throw std::logic_error("gmres before factorize");
        spand::PcgResult r = spand::device_gmres(*t->t->device(), t->t->device_csr(), b, x, iters, restart, tol);
        if (iters_out) *iters_out = r.iterations;
        if (relres_out) *relres_out = r.relres;
    });
}

int spand_fgmres(spand_tree* t, const double* b, double* x, int iters, int restart, double tol, int verb,
                 int* iters_out, double* relres_out) {
    CHECK_T(t);
    if (!b || !x) return fail(SPAND_ERR_ARG, "null vector");
    if (restart < 1) return fail(SPAND_ERR_ARG, "restart < 1");
    return guard([&] {
        double rr = 0;
        int it = spaND::fgmres(t->t->matrix(), b, x, *t->t, iters, restart, tol, verb != 0, &rr);
        if (iters_out) *iters_out = it;
        if (relres_out) *relres_out = rr;
    });
}

int spand_ir(spand_tree* t, const double* b, double* x, int iters, double tol, int verb, int* iters_out,
             double* relres_out) {
    CHECK_T(t);
    if (!b || !x) return fail(SPAND_ERR_ARG, "null vector");
    return guard([&] {
        double rr = 0;
        int it = spaND::ir(t->t->matrix(), b, x, *t->t, iters, tol, verb != 0, &rr);
        if (iters_out) *iters_out = it;
        if (relres_out) *relres_out = rr;
    });
}

int spand_cg_device(spand_tree* t, const double* b, double* x, int iters, double tol, int* iters_out,
                    double* relres_out) {
    CHECK_T(t);
    if (!b || !x) return fail(SPAND_ERR_ARG, "null vector");
    return guard([&] {
        if (!t->t->device()) throw std::logic_error("cg before factorize");
        spand::PcgResult r = spand::device_pcg(*t->t->device(), t->t->device_csr(), b, x, iters, tol, true);
        if (iters_out) *iters_out = r.iterations;
        if (relres_out) *relres_out = r.relres;
    });
}

int spand_adjoint_device(spand_tree* t, const double* g, const double* x, double* lambda, double* grad_vals,
                         int iters, double tol, int* iters_out, double* relres_out) {
    CHECK_T(t);
    if (!g || !x || !lambda || !grad_vals) return fail(SPAND_ERR_ARG, "null vector");
    return guard([&] {
        spand::PcgResult r = t->t->adjoint_device(g, x, lambda, grad_vals, iters, tol);
        if (iters_out) *iters_out = r.iterations;
        if (relres_out) *relres_out = r.relres;
    });
}

int spand_tree_assemble_values(spand_tree* t, const double* vals, long long nnz, int on_device) {
    CHECK_T(t);
    if (!vals && nnz > 0) return fail(SPAND_ERR_ARG, "null values");
    return guard([&] { t->t->assemble_values(vals, (int64_t)nnz, on_device != 0); });
}

int spand_batch_factorize(spand_tree* const* trees, int count, int* status_out) {
    if (!trees || !status_out || count < 0) return fail(SPAND_ERR_ARG, "null argument");
    std::vector<spaND::Tree*> ts(count);
    for (int k = 0; k < count; k++) {
        if (!trees[k]) return fail(SPAND_ERR_ARG, "null tree");
        ts[k] = trees[k]->t;
    }
    return guard([&] {
        std::vector<std::string> msg(count);
        spaND::batch_factorize(ts.data(), count, status_out, msg.data());
        std::string first;
        for (int k = 0; k < count; k++) {
            if (!status_out[k]) continue;
            const bool piv = msg[k].find("Non-SPD") != std::string::npos ||
                             msg[k].find("Singular Pivot") != std::string::npos;
            status_out[k] = piv ? SPAND_ERR_NOT_SPD : SPAND_ERR_CUDA;
            if (first.empty()) first = "tree " + std::to_string(k) + ": " + msg[k];
        }
        if (!first.empty()) throw std::runtime_error(first);
    });
}

int spand_batch_cg(spand_tree* const* trees, int count, const double* const* b, double* const* x, int iters,
                   double tol, int* iters_out, double* relres_out) {
    if (!trees || !b || !x || !iters_out || !relres_out || count < 0) return fail(SPAND_ERR_ARG, "null argument");
    std::vector<spaND::Tree*> ts(count);
    for (int k = 0; k < count; k++) {
        if (!trees[k] || !b[k] || !x[k]) return fail(SPAND_ERR_ARG, "null tree or vector");
        ts[k] = trees[k]->t;
    }
    return guard([&] { spaND::batch_cg(ts.data(), count, b, x, iters, tol, iters_out, relres_out); });
}

int spand_batch_cg_device(spand_tree* const* trees, int count, const double* const* b, double* const* x, int iters,
                          double tol, int* iters_out, double* relres_out) {
    if (!trees || !b || !x || !iters_out || !relres_out || count < 0) return fail(SPAND_ERR_ARG, "null argument");
    std::vector<spaND::Tree*> ts(count);
    for (int k = 0; k < count; k++) {
        if (!trees[k] || !b[k] || !x[k]) return fail(SPAND_ERR_ARG, "null tree or vector");
        ts[k] = trees[k]->t;
    }
    return guard([&] { spaND::batch_cg_device(ts.data(), count, b, x, iters, tol, iters_out, relres_out); });
}

int spand_cg_multi(spand_tree* t, const double* b, double* x, int nrhs, int ld, int iters, double tol,
                   int* iters_out, double* relres_out) {
    CHECK_T(t);
    if (!b || !x || !iters_out || !relres_out) return fail(SPAND_ERR_ARG, "null argument");
    if (nrhs < 0 || ld < 0) return fail(SPAND_ERR_ARG, "negative size");
    return guard([&] {
        if (!t->t->device()) throw std::logic_error("cg before factorize");
        spaND::cg_multi(*t->t, b, x, nrhs, ld, iters, tol, iters_out, relres_out);
    });
}

int spand_cg_multi_device(spand_tree* t, const double* b, double* x, int nrhs, int iters, double tol,
                          int* iters_out, double* relres_out) {
    CHECK_T(t);
    if (!b || !x || !iters_out || !relres_out) return fail(SPAND_ERR_ARG, "null argument");
    if (nrhs < 0) return fail(SPAND_ERR_ARG, "negative size");
    return guard([&] {
        if (!t->t->device()) throw std::logic_error("cg before factorize");
        if (nrhs > 0)
            spand::device_pcg_multi(*t->t->device(), t->t->device_csr(), b, x, nrhs, iters, tol, true, iters_out,
                                    relres_out);
    });
}

int spand_tree_get_N(spand_tree* t, int* n) { CHECK_T(t); *n = t->t->get_N(); return SPAND_OK; }
int spand_tree_get_perm(spand_tree* t, int* perm) {
    CHECK_T(t);
    const auto& p = t->t->get_assembly_perm();
    std::memcpy(perm, p.data(), p.size() * sizeof(int));
    return SPAND_OK;
}
int spand_tree_nnz(spand_tree* t, long long* nnz) { CHECK_T(t); *nnz = t->t->nnz(); return SPAND_OK; }
int spand_tree_get_stop(spand_tree* t, int* stop) { CHECK_T(t); *stop = t->t->get_stop(); return SPAND_OK; }
int spand_tree_level_log(spand_tree* t, long long* out) {
    CHECK_T(t);
    const auto& L = t->t->log();
    for (size_t l = 0; l < L.size(); l++) {
        long long* o = out + 11 * l;
        o[0] = L[l].dofs_nd; o[1] = L[l].dofs_left_nd; o[2] = L[l].dofs_left_elim; o[3] = L[l].dofs_left_spars;
        o[4] = L[l].rank_before_sum; o[5] = L[l].rank_after_sum; o[6] = L[l].rank_after_count; o[7] = L[l].ignored;
        o[8] = L[l].nbrs_sum; o[9] = L[l].nbrs_count; o[10] = L[l].fact_nnz;
    }
    return SPAND_OK;
}
int spand_tree_num_ranks(spand_tree* t, int* n) { CHECK_T(t); *n = (int)t->t->ranks().size(); return SPAND_OK; }
int spand_tree_get_ranks(spand_tree* t, int* out) {
    CHECK_T(t);
    auto r = t->t->ranks();
    for (size_t i = 0; i < r.size(); i++)
        for (int k = 0; k < 4; k++) out[4 * i + k] = r[i][k];
    return SPAND_OK;
}
int spand_tree_num_ops(spand_tree* t, int* n) { CHECK_T(t); *n = (int)t->t->ops().size(); return SPAND_OK; }
int spand_tree_get_ops(spand_tree* t, int* out) {
    CHECK_T(t);
    const auto& ops = t->t->ops();
    for (size_t i = 0; i < ops.size(); i++) {
        int* o = out + 8 * i;
        o[0] = ops[i].kind; o[1] = ops[i].level; o[2] = ops[i].self; o[3] = ops[i].nbr;
        o[4] = ops[i].ns; o[5] = ops[i].nn; o[6] = ops[i].rows; o[7] = ops[i].cols;
    }
    return SPAND_OK;
}
int spand_tree_get_op_matrix(spand_tree* t, int idx, double* out) {
    CHECK_T(t);
    return guard([&] {
        std::vector<double> m;
        t->t->op_matrix(idx, m);
        std::memcpy(out, m.data(), m.size() * sizeof(double));
    });
}
int spand_tree_get_op_signs(spand_tree* t, int idx, double* out) {
    CHECK_T(t);
    return guard([&] {
        std::vector<double> m;
        t->t->op_signs(idx, m);
        std::memcpy(out, m.data(), m.size() * sizeof(double));
    });
}
int spand_tree_get_op_perm(spand_tree* t, int idx, int* out) {
    CHECK_T(t);
    return guard([&] {
        std::vector<int> m;
        t->t->op_perm(idx, m);
        std::memcpy(out, m.data(), m.size() * sizeof(int));
    });
}
int spand_tree_get_op_tau(spand_tree* t, int idx, double* out) {
    CHECK_T(t);
    return guard([&] {
        std::vector<double> m;
        t->t->op_tau(idx, m);
        std::memcpy(out, m.data(), m.size() * sizeof(double));
    });
}
int spand_tree_timings(spand_tree* t, double* out) {
    CHECK_T(t);
    out[0] = t->t->t_partition; out[1] = t->t->t_assemble; out[2] = t->t->t_factorize;
    return SPAND_OK;
}
int spand_tree_launches(spand_tree* t, long long* n, int reset) {
    CHECK_T(t);
    *n = t->t->launches();
    if (reset) t->t->reset_launches();
    return SPAND_OK;
}
int spand_tree_device_bytes(spand_tree* t, long long* b) { CHECK_T(t); *b = (long long)t->t->device_bytes(); return SPAND_OK; }

int spand_tree_bench_step(spand_tree* t, const double* b, double* x, int nrhs, int iters, double tol, double* out) {
    CHECK_T(t);
    if (!b || !x || !out) return fail(SPAND_ERR_ARG, "null argument");
    if (nrhs < 1) return fail(SPAND_ERR_ARG, "nrhs < 1");
    return guard([&] { t->t->bench_step(b, x, nrhs, iters, tol, out); });
}
int spand_tree_assembled_bytes(spand_tree* t, long long* b) {
    CHECK_T(t);
    if (!t->t->device()) return fail(SPAND_ERR_STATE, "before assemble");
    *b = (long long)t->t->matrix().val.size() * (long long)sizeof(double);
    return SPAND_OK;
}
int spand_tree_set_profiling(spand_tree* t, int on) {
    CHECK_T(t);
    if (!t->t->device()) return fail(SPAND_ERR_STATE, "profiling before assemble");
    t->t->device()->profiler().enable(on != 0);
    return SPAND_OK;
}
int spand_tree_profile_count(spand_tree* t, int* n) {
    CHECK_T(t);
    if (!t->t->device()) return fail(SPAND_ERR_STATE, "profiling before assemble");
    return guard([&] {
        spand::DeviceScope scope(t->t->device_id());
        t->t->device()->profiler().collect();
        *n = (int)t->t->device()->profiler().totals().size();
    });
}
int spand_tree_profile_entry(spand_tree* t, int idx, char* name, long long* launches, double* ms) {
    CHECK_T(t);
    if (!t->t->device()) return fail(SPAND_ERR_STATE, "profiling before assemble");
    const auto& v = t->t->device()->profiler().totals();
    if (idx < 0 || idx >= (int)v.size()) return fail(SPAND_ERR_ARG, "index out of range");
    std::strncpy(name, v[idx].cls.c_str(), 63);
    name[63] = 0;
    *launches = v[idx].launches;
    *ms = v[idx].ms;
    return SPAND_OK;
}
int spand_tree_profile_reset(spand_tree* t) {
    CHECK_T(t);
    if (t->t->device()) t->t->device()->profiler().clear();
    return SPAND_OK;
}
int spand_tree_qrcp_wave_count(spand_tree* t, int* n) {
    CHECK_T(t);
    if (!n) return fail(SPAND_ERR_ARG, "null output");
    if (!t->t->device()) return fail(SPAND_ERR_STATE, "before assemble");
    *n = (int)t->t->device()->qrcp_waves().size();
    return SPAND_OK;
}
int spand_tree_qrcp_wave(spand_tree* t, int idx, int* conf9, int* ncand) {
    CHECK_T(t);
    if (!conf9 || !ncand) return fail(SPAND_ERR_ARG, "null output");
    if (!t->t->device()) return fail(SPAND_ERR_STATE, "before assemble");
    const auto v = t->t->device()->qrcp_waves();
    if (idx < 0 || idx >= (int)v.size()) return fail(SPAND_ERR_ARG, "index out of range");
    std::copy(v[idx].conf, v[idx].conf + 9, conf9);
    *ncand = (int)v[idx].cand.size();
    return SPAND_OK;
}
int spand_tree_qrcp_wave_candidate(spand_tree* t, int idx, int k, int* conf5, double* ms) {
    CHECK_T(t);
    if (!conf5 || !ms) return fail(SPAND_ERR_ARG, "null output");
    if (!t->t->device()) return fail(SPAND_ERR_STATE, "before assemble");
    const auto v = t->t->device()->qrcp_waves();
    if (idx < 0 || idx >= (int)v.size()) return fail(SPAND_ERR_ARG, "index out of range");
    if (k < 0 || k >= (int)v[idx].cand.size()) return fail(SPAND_ERR_ARG, "candidate out of range");
    std::copy(v[idx].cand[k].begin(), v[idx].cand[k].end(), conf5);
    *ms = v[idx].ms[k];
    return SPAND_OK;
}
int spand_tree_work_count(spand_tree* t, int which, int* n) {
    CHECK_T(t);
    return guard([&] { *n = (int)(which ? t->t->work_solve() : t->t->work_factor()).size(); });
}
int spand_tree_work_entry(spand_tree* t, int which, int idx, char* name, double* bytes, double* flops) {
    CHECK_T(t);
    return guard([&] {
        auto v = which ? t->t->work_solve() : t->t->work_factor();
        if (idx < 0 || idx >= (int)v.size()) throw std::invalid_argument("index out of range");
        std::strncpy(name, v[idx].cls.c_str(), 63);
        name[63] = 0;
        *bytes = v[idx].bytes;
        *flops = v[idx].flops;
    });
}

#define CHECK_F(f) \
    if (!(f) || !(f)->f) return fail(SPAND_ERR_ARG, "null forest")

int spand_forest_create(spand_forest** out, spand_tree* const* trees, int count) {
    if (!out || !trees || count <= 0) return fail(SPAND_ERR_ARG, "null argument");
    std::vector<spaND::Tree*> ts(count);
    for (int k = 0; k < count; k++) {
        if (!trees[k] || !trees[k]->t) return fail(SPAND_ERR_ARG, "null tree");
        ts[k] = trees[k]->t;
    }
    return guard([&] {
        auto* h = new spand_forest();
        try {
            h->f = new spaND::Forest(ts.data(), count);
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
    });
}

int spand_forest_destroy(spand_forest* f) {
    if (!f) return SPAND_OK;
    delete f->f;
    delete f;
    return SPAND_OK;
}

int spand_forest_offsets(spand_forest* f, long long* off, long long* nnz_off) {
    CHECK_F(f);
    if (off) std::memcpy(off, f->f->offsets().data(), f->f->offsets().size() * sizeof(long long));
    if (nnz_off)
        std::memcpy(nnz_off, f->f->value_offsets().data(), f->f->value_offsets().size() * sizeof(long long));
    return SPAND_OK;
}

int spand_forest_assemble_values(spand_forest* f, const double* vals, long long nnz, int on_device) {
    CHECK_F(f);
    if (!vals && nnz > 0) return fail(SPAND_ERR_ARG, "null values");
    return guard([&] { f->f->assemble_values(vals, (int64_t)nnz, on_device != 0); });
}

int spand_forest_factorize(spand_forest* f, int* failed_system) {
    CHECK_F(f);
    const int rc = guard([&] { f->f->factorize(); });
    if (failed_system) *failed_system = f->f->failed_system();
    return rc;
}

int spand_forest_solve_device(spand_forest* f, double* x) {
    CHECK_F(f);
    if (!x) return fail(SPAND_ERR_ARG, "null vector");
    return guard([&] { f->f->solve_device(x); });
}

int spand_forest_cg(spand_forest* f, const double* b, double* x, int iters, double tol, int* iters_out,
                    double* relres_out) {
    CHECK_F(f);
    if (!b || !x || !iters_out || !relres_out) return fail(SPAND_ERR_ARG, "null argument");
    return guard([&] { f->f->cg(b, x, iters, tol, iters_out, relres_out); });
}

int spand_forest_cg_device(spand_forest* f, const double* b, double* x, int iters, double tol, int* iters_out,
                           double* relres_out) {
    CHECK_F(f);
    if (!b || !x || !iters_out || !relres_out) return fail(SPAND_ERR_ARG, "null argument");
    return guard([&] { f->f->cg_device(b, x, iters, tol, iters_out, relres_out); });
}

int spand_forest_num_ranks(spand_forest* f, int* n) {
    CHECK_F(f);
    return guard([&] { *n = (int)f->f->ranks().size(); });
}

int spand_forest_get_ranks(spand_forest* f, int* out) {
    CHECK_F(f);
    return guard([&] {
        auto r = f->f->ranks();
        for (size_t i = 0; i < r.size(); i++)
            for (int j = 0; j < 5; j++) out[5 * i + j] = r[i][j];
    });
}

int spand_forest_set_profiling(spand_forest* f, int on) {
    CHECK_F(f);
    f->f->device()->profiler().enable(on != 0);
    return SPAND_OK;
}
int spand_forest_profile_count(spand_forest* f, int* n) {
    CHECK_F(f);
    return guard([&] {
        spand::DeviceScope scope(f->f->device_id());
        f->f->device()->profiler().collect();
        *n = (int)f->f->device()->profiler().totals().size();
    });
}
int spand_forest_profile_entry(spand_forest* f, int idx, char* name, long long* launches, double* ms) {
    CHECK_F(f);
    const auto& v = f->f->device()->profiler().totals();
    if (idx < 0 || idx >= (int)v.size()) return fail(SPAND_ERR_ARG, "index out of range");
    std::strncpy(name, v[idx].cls.c_str(), 63);
    name[63] = 0;
    *launches = v[idx].launches;
    *ms = v[idx].ms;
    return SPAND_OK;
}
int spand_forest_profile_reset(spand_forest* f) {
    CHECK_F(f);
    f->f->device()->profiler().clear();
    return SPAND_OK;
}

int spand_forest_launches(spand_forest* f, long long* n, int reset) {
    CHECK_F(f);
    if (n) *n = (long long)f->f->launches();
    if (reset) f->f->reset_launches();
    return SPAND_OK;
}

}  // extern "C"

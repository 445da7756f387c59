// C ABI of the evaluator: parameter resolution (autotuner), plans (device
// buffers, tables, twiddles, CUDA-graph replay), the one-shot solve and the
// reference-facing entry points.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "pb_internal.h"
#include "pb_kernel_math.h"
#include "pb_kernels.h"
#include "pbrinkman.h"

using namespace pb;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define PB_CK(call)                                                                              \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess) return fail(PB_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

bool finite(double v) { return std::isfinite(v); }

int pow2ceil(int v)
{
    int p = 8;
    while (p < v) p <<= 1;
    return p;
}

bool is_pow2(int v) { return v >= 4 && (v & (v - 1)) == 0; }

struct Resolved {
    double d, rc, eta, m, tol;
    int M[3];
    int P;
    int Pa[3];
    int nc[3], S[3];
    double h[3];
    int n_src, n_tgt;  // n_tgt: effective targets (n_src when targets are the sources)
    int same;
    int flags;
    long long pairs_est;
};

// Per-unit device costs (seconds) used by the splitting choice.
struct CostModel {
    double pair, grid, support;
};

// Per-unit device times measured on a GB300 (N = 1e5, 128^3, P = 12): mixed
// precision 0.65 ms / 42e6 pairs, 0.26 ms per 128^3 FFT round trip of three
// components, 0.79 ms / (2e5 x 1728) window points spread plus gathered.
// (The kernels have since become faster: 0.50 ms, 0.093 ms and 0.53 ms.  A
// model refitted to those figures picks finer grids for the serving stream
// and served 4% fewer solves/s with a higher p99, since grid clears, launch
// overhead and batching are not in it; the earlier constants are kept.)
CostModel cost_model(int prec)
{
    if (prec == PB_PREC_MIXED) return {1.5e-11, 1.2e-10, 2.3e-12};
    return {1.5e-10, 2.4e-10, 4.6e-12};
}

int validate(const pb_solve_params& p)
{
    if (p.n_src < 0 || p.n_tgt < 0) return fail(PB_ERR_INVALID, "negative particle count");
    for (int a = 0; a < 3; a++)
        if (!finite(p.L[a]) || !(p.L[a] > 0)) return fail(PB_ERR_INVALID, "box length L[%d] must be > 0", a);
    if (!finite(p.alpha) || !(p.alpha > 0)) return fail(PB_ERR_INVALID, "alpha must be > 0");
    if (!finite(p.eps) || p.eps < 0) return fail(PB_ERR_INVALID, "eps must be >= 0");
    if (!finite(p.tol) || p.tol < 0 || p.tol >= 1) return fail(PB_ERR_INVALID, "tol must be in [0, 1)");
    if (!finite(p.d) || p.d < 0) return fail(PB_ERR_INVALID, "d must be >= 0");
    if (!finite(p.rc) || p.rc < 0) return fail(PB_ERR_INVALID, "rc must be >= 0");
    if (!finite(p.m_std) || p.m_std < 0) return fail(PB_ERR_INVALID, "m_std must be >= 0");
    for (int a = 0; a < 3; a++)
        if (p.M[a] != 0 && (!is_pow2(p.M[a]) || p.M[a] < 8 || p.M[a] > 1024))
            return fail(PB_ERR_UNSUPPORTED, "grid M[%d]=%d: powers of two in [8, 1024] are supported", a, p.M[a]);
    if (p.P != 0 && (p.P < 4 || p.P > 32 || (p.P & 1)))
        return fail(PB_ERR_UNSUPPORTED, "support P=%d: even values in [4, 32] are supported", p.P);
    if (p.precision != PB_PREC_FP64 && p.precision != PB_PREC_MIXED) return fail(PB_ERR_INVALID, "bad precision");
    if (p.flags & ~(PB_REAL_SPACE | PB_KSPACE | PB_ZERO_MODE)) return fail(PB_ERR_INVALID, "bad flags");
    return PB_OK;
}

// Choose the grid for splitting width d (tuning fields the user left at 0).
// u = d/h is the splitting width in grid units that the Gaussian needs.
void grid_for(const pb_solve_params& p, double d, double u, double kconst, int* M)
{
    for (int a = 0; a < 3; a++) {
        if (p.M[a] > 0) {
            M[a] = p.M[a];
            continue;
        }
        // k-space truncation exp(-kmax^2 d^2/4) <= tol/10 with kmax = 2 pi (M/2 - 1)/L
        // (Nyquist planes are zeroed), and the spreading error bound on d/h
        double nk = 2.0 * std::sqrt(kconst) / d * p.L[a] / (2 * M_PI) + 1.0;
        double mk = 2.0 * nk + 2.0;
        double md = p.L[a] * u / d + 2.0;
        M[a] = pow2ceil((int)std::ceil(std::max(mk, md)));
    }
}

// Spectral-Ewald error model of the Gaussian support (s = eta/h^2 in grid units):
//   window truncation   exp(-(P/2 - 1)^2 / s)        (the window reaches (P/2-1) h)
//   aliasing            exp(-pi^2 s (1 - s h^2/d^2))  (worst mode after deconvolution)
// For a support P the widest admissible Gaussian minimises the d/h the
// aliasing bound asks for.
struct Support {
    int P;
    double s, u;  // u = minimal d/h
};

Support support_for(int P, double Ealias, double Etrunc, double m_std)
{
    Support S;
    S.P = P;
    if (m_std > 0) {
        S.s = (double)P * P / (2.0 * m_std * m_std);  // the reference's eta = (P h / m)^2 / 2
    } else {
        S.s = std::min(2.0 * Ealias / (M_PI * M_PI), (P / 2.0 - 1.0) * (P / 2.0 - 1.0) / Etrunc);
    }
    double ps = M_PI * M_PI * S.s;
    if (ps > 1.02 * Ealias)
        S.u = std::sqrt(ps * S.s / (ps - Ealias));
    else
        S.u = 1e9;  // this support cannot reach the tolerance
    return S;
}

int resolve(const pb_solve_params& p, Resolved& R)
{
    int rc_ = validate(p);
    if (rc_) return rc_;
    const double tol = p.tol > 0 ? p.tol : 1e-6;
    R.tol = tol;
    R.flags = p.flags ? p.flags : PB_FLAGS_DEFAULT;
    R.n_src = p.n_src;
    R.same = (p.n_tgt == 0);
    R.n_tgt = R.same ? p.n_src : p.n_tgt;
    // error budgets aim at tol/2 so that the sum of the parts stays below tol
    const double kconst = std::log(20.0 / tol);      // k-space truncation exponent
    // aliasing exponent; measured as the cutoff margin below: an offset of +1
    // gives 2.4e-7 (tol 1e-6) and 1.5e-5 (tol 1e-4) on the serving stream, 0
    // gives 2.9e-7 and 3.4e-5, -1 gives 2.5e-6 (above tol)
    const double ealias = std::log(2.0 / tol);
    const double etrunc = std::max(4.0, ealias - 3.0);
    // rc = zeta d.  Measured on the serving stream and the N = 1e5 solve (max
    // relative error of sampled requests against the FP64 oracle): an offset
    // of 0.35 gives 2e-7 at tol 1e-6 and 3.6e-6 at 1e-4; 0 gives 3.3e-7 and
    // 2.1e-5; -0.25 gives 1.6e-6 (above tol).  0.1 keeps a margin of about 3.
    const double zeta = std::sqrt(std::log(2.0 / tol)) + 0.1;
    const double uk = 2.0 * std::sqrt(kconst) / M_PI;  // d/h asked by the k-space truncation
    // candidate supports: the given one, else every even P that can reach the
    // tolerance; the splitting width and the support are chosen together for
    // the lowest modelled cost
    std::vector<Support> cands;
    if (p.P > 0) {
        Support t = support_for(p.P, ealias, etrunc, p.m_std);
        if (t.u > 1e8) t.u = uk;  // user support below the tolerance: keep the k-space bound
        cands.push_back(t);
    } else {
        for (int P = 6; P <= 32; P += 2) {
            Support t = support_for(P, ealias, etrunc, p.m_std);
            if (t.u < 1e8) cands.push_back(t);
        }
        if (cands.empty()) cands.push_back(support_for(32, ealias, etrunc, p.m_std));
    }
    const double tau = p.L[0] * p.L[1] * p.L[2];
    const double Lmin = std::min(p.L[0], std::min(p.L[1], p.L[2]));
    const CostModel C = cost_model(p.precision);
    auto real_cut = [&](double d) {
        double rc = p.rc > 0 ? p.rc : zeta * d;
        if (p.rc == 0 && p.eps > 0) rc = std::max(rc, zeta * p.eps);
        return rc;
    };
    double best = 1e300, d = p.d > 0 ? p.d : Lmin / 8;
    Support sup = cands.front();
    // modelled cost of (support, d); +inf when the grid or the fixed-grid limits exclude it
    auto cost_at = [&](const Support& cand, double dd) {
        const double u = std::max(cand.u, uk);
        int M[3];
        grid_for(p, dd, u, kconst, M);
        bool ok = true;
        for (int a = 0; a < 3; a++) {
            if (M[a] > 1024 || cand.P > M[a]) ok = false;
            if (p.M[a] > 0 && p.d == 0) {  // fixed grid: d must satisfy its k-space and spreading limits
                double kmax = 2 * M_PI * (M[a] / 2 - 1) / p.L[a];
                if (kmax * dd / 2 < std::sqrt(kconst)) ok = false;
                if (p.L[a] / M[a] * u > dd) ok = false;
            }
        }
        if (!ok && !(p.d > 0 && cands.size() == 1)) return 1e300;
        double rc = real_cut(dd);
        double pairs = (double)R.n_tgt * p.n_src * (4 * M_PI / 3) * rc * rc * rc / tau;
        double grid = (double)M[0] * M[1] * M[2];
        if ((R.flags & PB_KSPACE) == 0) return C.pair * pairs;
        return C.pair * pairs + C.grid * grid * std::log2(std::max(grid, 2.0)) / 21.0 +
               C.support * (double)(p.n_src + R.n_tgt) * cand.P * cand.P * cand.P;
    };
    auto consider = [&](const Support& cand, double dd) {
        const double c = cost_at(cand, dd);
        if (c < best) {
            best = c;
            d = dd;
            sup = cand;
        }
        return c;
    };
    // the smallest supports that reach the tolerance (larger ones only add window points)
    if (cands.size() > 4) cands.resize(4);
    for (const Support& cand : cands) {
        if (p.d > 0) {
            consider(cand, p.d);
            continue;
        }
        // d = Lmin 2^(-1 - k/16): a coarse pass every 4th k, then the fine steps around its best
        double cbest = 1e300;
        int kbest = 0;
        for (int k = 0; k < 160; k += 4) {
            const double dd = Lmin * std::pow(2.0, -1.0 - k * 0.0625);
            if (dd < 1e-6) break;
            const double c = consider(cand, dd);
            if (c < cbest) {
                cbest = c;
                kbest = k;
            }
        }
        for (int k = std::max(0, kbest - 8); k <= std::min(159, kbest + 8); k++) {
            const double dd = Lmin * std::pow(2.0, -1.0 - k * 0.0625);
            if (dd >= 1e-6) consider(cand, dd);
        }
    }
    const int P = sup.P;
    const double s = sup.s;
    const double u = std::max(sup.u, uk);
    R.P = P;
    R.m = P / std::sqrt(2.0 * s);
    R.d = d;
    R.rc = real_cut(d);
    grid_for(p, d, u, kconst, R.M);
    for (int a = 0; a < 3; a++)
        if (R.M[a] > 1024)
            return fail(PB_ERR_UNSUPPORTED, "grid %d needed along axis %d exceeds 1024", R.M[a], a);
    for (int a = 0; a < 3; a++)
        if (R.P > R.M[a]) return fail(PB_ERR_UNSUPPORTED, "support P=%d exceeds grid M[%d]=%d", R.P, a, R.M[a]);
    // eta from the coarsest axis (aliasing); finer axes get more support points
    // so that every axis reaches the same truncation exponent
    double hmax = std::max(p.L[0] / R.M[0], std::max(p.L[1] / R.M[1], p.L[2] / R.M[2]));
    R.eta = s * hmax * hmax;
    for (int a = 0; a < 3; a++) {
        double h = p.L[a] / R.M[a];
        int Pa = R.P;
        if (p.m_std == 0) Pa = std::max(R.P, 2 * (int)std::ceil(std::sqrt(etrunc * R.eta) / h + 1.0));
        if (Pa > 32) return fail(PB_ERR_UNSUPPORTED, "anisotropic grid needs support %d > 32 along axis %d", Pa, a);
        if (Pa > R.M[a]) return fail(PB_ERR_UNSUPPORTED, "support %d exceeds grid M[%d]=%d", Pa, a, R.M[a]);
        R.Pa[a] = Pa;
    }
    // cell list: cells at least rc/2 wide across (two-cell reach) and rc/4 along z,
    // where each stencil column is cut to the part of the cutoff ball it meets;
    // capped at 128 per axis
    for (int a = 0; a < 3; a++) {
        int nc = (int)std::floor((a == 2 ? 4.0 : 2.0) * p.L[a] / R.rc);
        nc = std::max(1, std::min(128, nc));
        R.nc[a] = nc;
        R.h[a] = p.L[a] / nc;
        R.S[a] = (int)std::ceil(R.rc / R.h[a] - 1e-12);
        if (R.S[a] > 15) return fail(PB_ERR_UNSUPPORTED, "real-space cutoff spans more than 15 cells along axis %d", a);
    }
    R.pairs_est = (long long)((double)R.n_tgt * p.n_src * (4 * M_PI / 3) * R.rc * R.rc * R.rc / tau);
    return PB_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// Plans
// ---------------------------------------------------------------------------
struct Bucket {
    int M[3];
    std::vector<int> inst;
    int* d_inst = nullptr;
    void* d_tw = nullptr;
};

struct pb_plan_s {
    int count = 0, prec = 0, dev = 0, nsm = 148;
    bool all_same = true, any_real = false, any_k = false, any_zero = false;
    std::vector<pb_solve_params> par;
    std::vector<Resolved> res;
    std::vector<PbInst> hinst;
    std::vector<PbTables> htab;
    std::vector<int> src_off, tgt_off, cell_off, y_off;
    int n_src = 0, n_tgt = 0, ncell = 0, npoly = 16, n_y = 0;
    std::vector<Bucket> buckets;
    size_t grid_elems = 0, spec_elems = 0;

    char* arena = nullptr;
    size_t arena_bytes = 0;
    PbInst* d_inst = nullptr;
    PbTables* d_tab = nullptr;
    int *d_src_off = nullptr, *d_tgt_off = nullptr, *d_cell_off = nullptr, *d_y_off = nullptr;
    double *x = nullptr, *f = nullptr, *y = nullptr, *U = nullptr;
    // cell lists: per particle (cell, arrival slot); counts, scan flags and tickets (zeroed before
    // every build); starts of the source cells and, cell_list_stride apart, of the target cells
    int4 *key_s = nullptr, *key_t = nullptr;
    int *cl_zero = nullptr, *start_s = nullptr, *start_t = nullptr;
    size_t cl_zero_bytes = 0;
    int2 *perm_tmp_s = nullptr, *perm_tmp_t = nullptr;
    int *perm_s = nullptr, *perm_t = nullptr;
    int* counter = nullptr;
    int4* items = nullptr;
    void *spos_a = nullptr, *spos_b = nullptr, *sfrc = nullptr, *tpos_a = nullptr, *tpos_b = nullptr;
    double *u_real = nullptr, *fsum = nullptr;
    // per instance: an input was not finite (set by the binning kernels); entry
    // [count]: capacity bits of the execution (kCapItems: the real-space work
    // items outgrew the item array, so items were dropped)
    int* d_bad = nullptr;
    int* h_bad = nullptr;     // pinned copy, written at the end of every execution
    int item_cap = 0;         // capacity of the real-space work item array
    void *u_k = nullptr, *grid = nullptr, *spec = nullptr;

    // binding: a plan is a capacity; pb_plan_bind places actual instances in it
    int npoly_cap = 0;        // polynomial terms compiled into the captured real-space kernel
    int bound = 0;            // instances bound (<= count)
    int act_src = 0, act_tgt = 0, act_y = 0;
    bool upload_pending = false;
    char* staging = nullptr;  // pinned host copy of instances, tables and offsets
    size_t staging_bytes = 0;
    cudaEvent_t ev_upload = nullptr;

    cudaStream_t stream = nullptr;
    cudaStream_t stream_k = nullptr;  // the k-space branch of an execution (forked after the cell lists)
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    cudaGraphExec_t gexec = nullptr;
    cudaGraphExec_t gexec_f = nullptr;  // forces-only executions (positions of the last full one)
    int exec_count = 0;
    int fexec_count = 0;
    bool have_positions = false;  // a full execution since the last bind sorted the current positions
    int graph_kernels = 0;  // kernel nodes in the captured graph
    bool timing = false;
    cudaEvent_t tev[7] = {};
    double stage_ms[6] = {};
};

namespace {

size_t align_up(size_t v) { return (v + 255) & ~(size_t)255; }

struct Layout {
    size_t off = 0;
    template <class T>
    size_t take(size_t n)
    {
        size_t o = off;
        off += align_up(n * sizeof(T) + 16);
        return o;
    }
};

// Plan sizes; fills offsets when `P` has an arena.
size_t plan_layout(pb_plan_s* P, bool assign)
{
    Layout L;
    const bool mixed = P->prec == PB_PREC_MIXED;
    const int ns = std::max(P->n_src, 1), nt = std::max(P->n_tgt, 1), nc = std::max(P->ncell, 1);
    const int q = P->count;
    size_t o_inst = L.take<PbInst>(q), o_tab = L.take<PbTables>(q);
    size_t o_so = L.take<int>(q + 1), o_to = L.take<int>(q + 1), o_co = L.take<int>(q + 1), o_yo = L.take<int>(q + 1);
    size_t o_x = L.take<double>(3 * (size_t)ns), o_f = L.take<double>(3 * (size_t)ns);
    size_t o_y = P->all_same ? 0 : L.take<double>(3 * (size_t)std::max(P->n_y, 1));
    size_t o_U = L.take<double>(3 * (size_t)nt);
    const size_t zero_bytes = cell_list_zero_bytes(nc);
    size_t o_ks = L.take<int4>(ns), o_clz = L.take<char>(zero_bytes), o_sts = L.take<int>(2 * (size_t)cell_list_stride(nc)),
           o_ps = L.take<int>(ns), o_pts = L.take<int2>(ns);
    size_t o_kt = 0, o_pt = 0, o_ptt = 0;
    if (!P->all_same) {
        o_kt = L.take<int4>(nt);
        o_pt = L.take<int>(nt);
        o_ptt = L.take<int2>(nt);
    }
    const int item_cap = 4 * nt + 4096;
    size_t o_cnt = L.take<int>(4), o_it = L.take<int4>(item_cap);
    size_t o_sa, o_sb = 0, o_sf, o_ta = 0, o_tb = 0;
    if (mixed) {
        o_sa = L.take<float4>(ns);
        o_sb = L.take<float4>(ns);
        o_sf = L.take<float4>(ns);
        if (!P->all_same) {
            o_ta = L.take<float4>(nt);
            o_tb = L.take<float4>(nt);
        }
    } else {
        o_sa = L.take<Dbl4>(ns);
        o_sf = L.take<Dbl4>(ns);
        if (!P->all_same) o_ta = L.take<Dbl4>(nt);
    }
    size_t o_ur = L.take<double>(3 * (size_t)nt);
    size_t o_uk = mixed ? L.take<float>(3 * (size_t)nt) : L.take<double>(3 * (size_t)nt);
    size_t o_fsum = L.take<double>(3 * (size_t)q), o_bad = L.take<int>(q + 1);
    size_t esz = mixed ? 4 : 8;
    size_t o_grid = L.off;
    L.off += align_up(P->grid_elems * esz + 16);
    size_t o_spec = L.off;
    L.off += align_up(P->spec_elems * 2 * esz + 16);
    std::vector<size_t> o_tw(P->buckets.size()), o_bi(P->buckets.size());
    for (size_t b = 0; b < P->buckets.size(); b++) {
        o_tw[b] = L.off;
        L.off += align_up(twiddle_bytes(P->buckets[b].M, !mixed) + 16);
        o_bi[b] = L.take<int>(P->buckets[b].inst.size());
    }
    if (assign) {
        char* A = P->arena;
        P->d_inst = (PbInst*)(A + o_inst);
        P->d_tab = (PbTables*)(A + o_tab);
        P->d_src_off = (int*)(A + o_so);
        P->d_tgt_off = (int*)(A + o_to);
        P->d_cell_off = (int*)(A + o_co);
        P->d_y_off = (int*)(A + o_yo);
        P->x = (double*)(A + o_x);
        P->f = (double*)(A + o_f);
        P->y = P->all_same ? nullptr : (double*)(A + o_y);
        P->U = (double*)(A + o_U);
        P->key_s = (int4*)(A + o_ks);
        P->cl_zero = (int*)(A + o_clz);
        P->cl_zero_bytes = zero_bytes;
        P->start_s = (int*)(A + o_sts);
        P->perm_s = (int*)(A + o_ps);
        P->perm_tmp_s = (int2*)(A + o_pts);
        if (!P->all_same) {
            P->key_t = (int4*)(A + o_kt);
            P->start_t = P->start_s + cell_list_stride(nc);
            P->perm_t = (int*)(A + o_pt);
            P->perm_tmp_t = (int2*)(A + o_ptt);
        } else {
            P->key_t = nullptr;
            P->start_t = P->start_s;
            P->perm_t = P->perm_s;
            P->perm_tmp_t = nullptr;
        }
        P->counter = (int*)(A + o_cnt);
        P->items = (int4*)(A + o_it);
        P->spos_a = A + o_sa;
        P->spos_b = mixed ? (void*)(A + o_sb) : nullptr;
        P->sfrc = A + o_sf;
        if (P->all_same) {
            P->tpos_a = P->spos_a;
            P->tpos_b = P->spos_b;
        } else {
            P->tpos_a = A + o_ta;
            P->tpos_b = mixed ? (void*)(A + o_tb) : nullptr;
        }
        P->u_real = (double*)(A + o_ur);
        P->item_cap = item_cap;

        P->u_k = A + o_uk;
        P->fsum = (double*)(A + o_fsum);
        P->d_bad = (int*)(A + o_bad);
        P->grid = A + o_grid;
        P->spec = A + o_spec;
        for (size_t b = 0; b < P->buckets.size(); b++) {
            P->buckets[b].d_tw = A + o_tw[b];
            P->buckets[b].d_inst = (int*)(A + o_bi[b]);
        }
    }
    return L.off;
}

// Cells along z of a real-space work item.  Short items give a small
// instance enough items to spread over the GPU; long ones let sparse targets
// (a target set half the size of the sources holds about one target per
// cell) fill the 32 lanes of a warp, and a lane's candidates per target fall
// as the item's box lengthens.  Fitted on 300 requests of the serving stream
// (N log-uniform in [1e3, 2e5], targets N/2), each solved alone: the
// real-space sum took 38.1 ms at 8 cells for all, 34.5 ms by this rule, 34.1
// ms at the best span of every request.
int item_cells(const Resolved& R)
{
    const long long nt = R.n_tgt;
    const double tpc = (double)nt / std::max(1.0, (double)R.nc[0] * R.nc[1] * R.nc[2]);
    const int z = nt < 2000 ? 4 : nt < 5000 ? 8 : nt < 10000 ? 12 : nt < 30000 ? 16 : (tpc < 1.2 ? 32 : 24);
    return std::min(kItemCells, z);
}

// Per-instance descriptor fields from the resolved parameters
// (grid_off/spec_off/bucket are kept).
void set_inst_fields(PbInst& I, const pb_solve_params& p, const Resolved& R, int src_off, int tgt_off, int cell_off)
{
    for (int a = 0; a < 3; a++) {
        I.L[a] = p.L[a];
        I.h[a] = R.h[a];
        I.gh[a] = p.L[a] / R.M[a];
        I.gih[a] = R.M[a] / p.L[a];
        I.iL[a] = 1.0 / p.L[a];
        I.ih[a] = 1.0 / R.h[a];
        I.nc[a] = R.nc[a];
        I.S[a] = R.S[a];
        I.M[a] = R.M[a];
        I.zero_mode[a] = 0;
    }
    I.alpha = p.alpha;
    I.eps = p.eps;
    I.d = R.d;
    I.rc = R.rc;
    I.eta = R.eta;
    for (int a = 0; a < 3; a++) {
        I.ghh[a] = (float)I.gh[a];
        I.ghl[a] = (float)(I.gh[a] - (double)I.ghh[a]);
        I.gihf[a] = (float)I.gih[a];
    }
    I.inv_eta_f = (float)(1.0 / R.eta);
    for (int a = 0; a < 3; a++) {
        I.hch[a] = (float)R.h[a];
        I.hcl[a] = (float)(R.h[a] - (double)I.hch[a]);
        I.Lh[a] = (float)p.L[a];
        I.Ll[a] = (float)(p.L[a] - (double)I.Lh[a]);
    }
    double Mtot = (double)R.M[0] * R.M[1] * R.M[2];
    I.kfac = I.gh[0] * I.gh[1] * I.gh[2] / (Mtot * std::pow(M_PI * R.eta, 3.0));
    I.P = std::max(R.Pa[0], std::max(R.Pa[1], R.Pa[2]));
    for (int a = 0; a < 3; a++) I.Pa[a] = R.Pa[a];
    I.n_src = R.n_src;
    I.n_tgt = R.n_tgt;
    I.src_off = src_off;
    I.tgt_off = tgt_off;
    I.cell_off = cell_off;
    I.ncell = R.nc[0] * R.nc[1] * R.nc[2];
    I.flags = R.flags;
    I.same = R.same;
    I.csplit = 1;  // assign_splits() refines this per batch
    I.zspan = item_cells(R);
}

// Per-instance descriptor and tables (grid_off/spec_off/bucket are kept).
int fill_instance(pb_plan_s* P, int q, const pb_solve_params& p, const Resolved& R, int src_off, int tgt_off,
                  int cell_off, int max_terms)
{
    set_inst_fields(P->hinst[q], p, R, src_off, tgt_off, cell_off);
    int trc = build_tables(p.alpha, R.d, p.eps, R.rc, kTableTol, &P->htab[q], max_terms, p.precision == PB_PREC_FP64);
    if (trc) return fail(PB_ERR_INVALID, "table construction failed");
    return PB_OK;
}

// Real-space work items per row item (csplit) of the first `count` instances.
// A row item of a small instance carries a long candidate loop; splitting its
// stencil columns into groups gives the GPU enough items to stay busy and
// evens out the end of the dynamic item schedule.  The target is about 12160
// items' worth of equal work (five per resident warp of a GB300), bounded by
// the stencil columns and by the item array's capacity.  Measured on the
// N = 1e5 solve (real-space sum): 4864 items 0.40 ms, 7296 0.35, 12160 0.345,
// 19456 0.36, 38912 0.38 ms.
void assign_splits(pb_plan_s* P, int count)
{
    double W = 0;
    for (int q = 0; q < count; q++) W += std::max(1.0, (double)P->res[q].pairs_est);
    std::vector<int> G(count, 1);
    std::vector<long long> bound(count, 0);
    long long base = 0, extra = 0;
    for (int q = 0; q < count; q++) {
        const Resolved& R = P->res[q];
        const int ncol = (2 * R.S[0] + 1) * (2 * R.S[1] + 1);
        const double per_item = 24.0 * std::max(1.0, (double)R.pairs_est) / std::max(1, R.n_tgt);
        long long g = std::llround(per_item * 12160.0 / W);
        G[q] = (int)std::max(1LL, std::min<long long>(g, std::min(ncol, 255)));
        // items of an instance <= min(targets, cells + targets/32 + 1) row items
        const long long nc = (long long)R.nc[0] * R.nc[1] * R.nc[2];
        bound[q] = std::min<long long>(R.n_tgt, nc + R.n_tgt / 32 + 1);
        base += bound[q];
        extra += bound[q] * (G[q] - 1);
    }
    const long long room = (long long)P->item_cap - base;
    if (extra > room) {
        for (int q = 0; q < count; q++)
            G[q] = 1 + (int)((long long)(G[q] - 1) * std::max(0LL, room) / extra);
    }
    for (int q = 0; q < count; q++) P->hinst[q].csplit = G[q];
    for (int q = count; q < (int)P->hinst.size(); q++) P->hinst[q].csplit = 1;
}

int build_plan_host(const pb_solve_params* p, int count, pb_plan_s* P)
{
    if (count <= 0) return fail(PB_ERR_INVALID, "count must be >= 1");
    P->count = count;
    P->prec = p[0].precision;
    P->par.assign(p, p + count);
    P->res.resize(count);
    P->hinst.resize(count);
    P->htab.resize(count);
    P->src_off.assign(count + 1, 0);
    P->tgt_off.assign(count + 1, 0);
    P->cell_off.assign(count + 1, 0);
    P->y_off.assign(count + 1, -1);
    P->all_same = true;
    for (int q = 0; q < count; q++) {
        if (p[q].precision != P->prec) return fail(PB_ERR_INVALID, "all instances of a plan share one precision");
        int rc = resolve(p[q], P->res[q]);
        if (rc) return rc;
        if (!P->res[q].same) P->all_same = false;
    }
    long long ns = 0, nt = 0, nc = 0, ny = 0;
    for (int q = 0; q < count; q++) {
        const Resolved& R = P->res[q];
        P->src_off[q] = (int)ns;
        P->tgt_off[q] = (int)nt;
        P->cell_off[q] = (int)nc;
        if (!R.same) {
            P->y_off[q] = (int)ny;
            ny += R.n_tgt;
        }
        ns += R.n_src;
        nt += R.n_tgt;
        nc += (long long)R.nc[0] * R.nc[1] * R.nc[2];
    }
    if (ns > (1LL << 30) || nt > (1LL << 30) || nc > (1LL << 30))
        return fail(PB_ERR_UNSUPPORTED, "batch too large");
    P->src_off[count] = (int)ns;
    P->tgt_off[count] = (int)nt;
    P->cell_off[count] = (int)nc;
    P->n_src = (int)ns;
    P->n_tgt = (int)nt;
    P->ncell = (int)nc;
    P->n_y = (int)ny;
    // FFT buckets by grid size; grids/spectra contiguous per bucket
    P->grid_elems = 0;
    P->spec_elems = 0;
    P->any_real = P->any_k = P->any_zero = false;
    for (int q = 0; q < count; q++) {
        const Resolved& R = P->res[q];
        if (R.flags & PB_REAL_SPACE) P->any_real = true;
        if (R.flags & PB_KSPACE) P->any_k = true;
        if (R.flags & PB_ZERO_MODE) P->any_zero = true;
        int b = -1;
        for (size_t k = 0; k < P->buckets.size(); k++)
            if (!std::memcmp(P->buckets[k].M, R.M, sizeof(R.M))) b = (int)k;
        if (b < 0) {
            Bucket B;
            std::memcpy(B.M, R.M, sizeof(R.M));
            P->buckets.push_back(B);
            b = (int)P->buckets.size() - 1;
        }
        P->buckets[b].inst.push_back(q);
    }
    for (size_t b = 0; b < P->buckets.size(); b++) {
        Bucket& B = P->buckets[b];
        size_t gsz = (size_t)B.M[0] * B.M[1] * B.M[2], ssz = (size_t)B.M[0] * B.M[1] * (B.M[2] / 2 + 1);
        for (int q : B.inst) {
            PbInst& I = P->hinst[q];
            I.grid_off = (long long)P->grid_elems;
            I.spec_off = (long long)P->spec_elems;
            I.bucket = (int)b;
            P->grid_elems += 4 * gsz;
            P->spec_elems += 3 * ssz;
        }
    }
    if (!P->any_k) P->grid_elems = P->spec_elems = 0;
    int npoly = 16;
    for (int q = 0; q < count; q++) {
        int trc = fill_instance(P, q, p[q], P->res[q], P->src_off[q], P->tgt_off[q], P->cell_off[q], 0);
        if (trc) return trc;
        npoly = std::max(npoly, P->htab[q].nd);
    }
    P->npoly = npoly;
    P->npoly_cap = npoly;
    P->item_cap = 4 * std::max(P->n_tgt, 1) + 4096;  // as plan_layout sizes it
    assign_splits(P, count);
    P->bound = count;
    P->act_src = P->n_src;
    P->act_tgt = P->n_tgt;
    P->act_y = P->n_y;
    return PB_OK;
}

void plan_free(pb_plan_s* P)
{
    if (!P) return;
    if (P->gexec) cudaGraphExecDestroy(P->gexec);
    if (P->gexec_f) cudaGraphExecDestroy(P->gexec_f);
    if (P->arena) cudaFree(P->arena);
    if (P->staging) cudaFreeHost(P->staging);
    if (P->h_bad) cudaFreeHost(P->h_bad);
    if (P->ev_upload) cudaEventDestroy(P->ev_upload);
    if (P->ev_in) cudaEventDestroy(P->ev_in);
    if (P->ev_out) cudaEventDestroy(P->ev_out);
    for (auto& e : P->tev)
        if (e) cudaEventDestroy(e);
    if (P->ev_fork) cudaEventDestroy(P->ev_fork);
    if (P->ev_join) cudaEventDestroy(P->ev_join);
    if (P->stream_k) cudaStreamDestroy(P->stream_k);
    if (P->stream) cudaStreamDestroy(P->stream);
    delete P;
}

int plan_alloc(pb_plan_s* P)
{
    PB_CK(cudaGetDevice(&P->dev));
    PB_CK(cudaDeviceGetAttribute(&P->nsm, cudaDevAttrMultiProcessorCount, P->dev));
    P->arena_bytes = plan_layout(P, false);
    cudaError_t e = cudaMalloc(&P->arena, P->arena_bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        P->arena = nullptr;
        return fail(PB_ERR_NOMEM, "device allocation of %zu bytes failed: %s", P->arena_bytes, cudaGetErrorString(e));
    }
    plan_layout(P, true);
    PB_CK(cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking));
    PB_CK(cudaStreamCreateWithFlags(&P->stream_k, cudaStreamNonBlocking));
    PB_CK(cudaEventCreateWithFlags(&P->ev_fork, cudaEventDisableTiming));
    PB_CK(cudaEventCreateWithFlags(&P->ev_join, cudaEventDisableTiming));
    P->staging_bytes = (sizeof(PbInst) + sizeof(PbTables)) * (size_t)P->count + 4 * sizeof(int) * (P->count + 1);
    PB_CK(cudaMallocHost(&P->staging, P->staging_bytes));
    PB_CK(cudaMallocHost(&P->h_bad, sizeof(int) * (P->count + 1)));
    std::memset(P->h_bad, 0, sizeof(int) * (P->count + 1));
    PB_CK(cudaEventCreateWithFlags(&P->ev_upload, cudaEventDisableTiming));
    PB_CK(cudaEventCreateWithFlags(&P->ev_in, cudaEventDisableTiming));
    PB_CK(cudaEventCreateWithFlags(&P->ev_out, cudaEventDisableTiming));
    for (auto& ev : P->tev) PB_CK(cudaEventCreate(&ev));
    // static data
    PB_CK(cudaMemcpy(P->d_inst, P->hinst.data(), sizeof(PbInst) * P->count, cudaMemcpyHostToDevice));
    PB_CK(cudaMemcpy(P->d_tab, P->htab.data(), sizeof(PbTables) * P->count, cudaMemcpyHostToDevice));
    PB_CK(cudaMemcpy(P->d_src_off, P->src_off.data(), sizeof(int) * (P->count + 1), cudaMemcpyHostToDevice));
    PB_CK(cudaMemcpy(P->d_tgt_off, P->tgt_off.data(), sizeof(int) * (P->count + 1), cudaMemcpyHostToDevice));
    PB_CK(cudaMemcpy(P->d_cell_off, P->cell_off.data(), sizeof(int) * (P->count + 1), cudaMemcpyHostToDevice));
    PB_CK(cudaMemcpy(P->d_y_off, P->y_off.data(), sizeof(int) * (P->count + 1), cudaMemcpyHostToDevice));
    const bool fp64 = P->prec == PB_PREC_FP64;
    for (auto& B : P->buckets) {
        std::vector<char> tw(twiddle_bytes(B.M, fp64));
        fill_twiddles(B.M, fp64, tw.data());
        PB_CK(cudaMemcpy(B.d_tw, tw.data(), tw.size(), cudaMemcpyHostToDevice));
        PB_CK(cudaMemcpy(B.d_inst, B.inst.data(), sizeof(int) * B.inst.size(), cudaMemcpyHostToDevice));
    }
    return PB_OK;
}

// Cell lists and sorted records of the sources and (when they have their own)
// the targets.
void build_cell_lists(pb_plan_s* P, cudaStream_t s)
{
    cudaMemsetAsync(P->cl_zero, 0, P->cl_zero_bytes, s);
    CellListArgs a;
    a.x = P->x;
    a.f = P->f;
    a.y = P->y;
    a.src_off = P->d_src_off;
    a.tgt_off = P->d_tgt_off;
    a.y_off = P->d_y_off;
    a.cell_off = P->d_cell_off;
    a.inst = P->d_inst;
    a.ninst = P->count;
    a.ncap_s = P->n_src;
    a.ncap_t = P->all_same ? 0 : P->n_tgt;
    a.two = P->all_same ? 0 : 1;
    a.ncell_cap = std::max(P->ncell, 1);
    a.key_s = P->key_s;
    a.key_t = P->key_t;
    a.zero = P->cl_zero;
    a.start = P->start_s;
    a.perm_tmp_s = P->perm_tmp_s;
    a.perm_tmp_t = P->perm_tmp_t;
    a.perm_s = P->perm_s;
    a.perm_t = P->perm_t;
    a.spos_a = P->spos_a;
    a.spos_b = P->spos_b;
    a.sfrc = P->sfrc;
    a.tpos_a = P->tpos_a;
    a.tpos_b = P->tpos_b;
    a.bad = P->d_bad;
    launch_cell_lists(a, P->prec == PB_PREC_MIXED, P->nsm, s);
}

// PB_SPREAD=atomic selects the point-wise spreading kernel (with a grid
// clear) in place of the tiled one, for comparing the two.
bool spread_atomic()
{
    static const bool v = [] {
        const char* e = std::getenv("PB_SPREAD");
        return e && std::strcmp(e, "atomic") == 0;
    }();
    return v;
}

void record(pb_plan_s* P, int k, cudaStream_t s)
{
    if (P->timing) cudaEventRecord(P->tev[k], s);
}

// The device work of one execution (inputs already in P->x/f/y).  With
// `forces_only` the cell lists, target records and work items of the last
// full execution are kept: only the source records are rebuilt (same
// positions, new forces).
void run_compute(pb_plan_s* P, cudaStream_t s, bool forces_only)
{
    const bool mixed = P->prec == PB_PREC_MIXED;
    NvtxRange nv_all("pb.compute");
    record(P, 0, s);
    cudaMemsetAsync(P->d_bad, 0, sizeof(int) * (P->count + 1), s);
    if (forces_only) {  // the source records again, in the sorted order of the last full execution
        if (mixed)
            launch_prepare_mixed(P->x, P->f, P->perm_s, P->n_src, P->d_src_off, P->d_inst, P->count,
                                 (float4*)P->spos_a, (float4*)P->spos_b, (float4*)P->sfrc, P->d_bad, s);
        else
            launch_prepare_fp64(P->x, P->f, P->perm_s, P->n_src, P->d_src_off, P->d_inst, P->count,
                                (Dbl4*)P->spos_a, (Dbl4*)P->sfrc, P->d_bad, s);
    } else {
        build_cell_lists(P, s);
    }
    if (!forces_only)
        launch_build_items(P->start_t, P->ncell, P->d_cell_off, P->d_inst, P->count, P->items, P->item_cap,
                           P->counter + 1, P->d_bad + P->count, P->nsm, s);
    record(P, 1, s);
    auto real_part = [&](cudaStream_t rs) {
        NvtxRange nv("pb.real_space");
        if (!P->any_real) return;
        const int* nitems = P->counter + 1;
        if (mixed)
            launch_real_mixed(P->npoly, P->d_inst, P->d_tab, P->items, nitems, P->item_cap,
                              (const float4*)P->spos_a, (const float4*)P->spos_b, (const float4*)P->sfrc, P->start_s,
                              (const float4*)P->tpos_a, (const float4*)P->tpos_b, P->n_tgt, P->u_real, P->counter,
                              P->nsm, rs);
        else
            launch_real_fp64(P->d_inst, P->d_tab, P->items, nitems, P->item_cap, (const Dbl4*)P->spos_a,
                             (const Dbl4*)P->sfrc, P->start_s, (const Dbl4*)P->tpos_a, P->n_tgt, P->u_real,
                             P->counter, P->nsm, rs);
    };
    auto kspace_part = [&](cudaStream_t ks) {
        NvtxRange nv("pb.kspace");
        if (!P->any_k) {
            record(P, 3, ks);
            record(P, 4, ks);
            return;
        }
        if (mixed && !spread_atomic()) {
            for (auto& B : P->buckets)
                launch_spread_tiles(P->d_inst, B.d_inst, (int)B.inst.size(), B.M, P->start_s, (const float4*)P->spos_a,
                                    (const float4*)P->spos_b, (const float4*)P->sfrc, (float*)P->grid, ks);
        } else if (mixed) {
            launch_zero_grids(P->d_inst, P->count, P->grid, 4, ks);
            launch_spread<float>(P->d_inst, P->count, P->d_src_off, P->n_src, P->spos_a, P->spos_b, P->sfrc,
                                 (float*)P->grid, ks);
        } else {
            launch_zero_grids(P->d_inst, P->count, P->grid, 8, ks);
            launch_spread<double>(P->d_inst, P->count, P->d_src_off, P->n_src, P->spos_a, P->spos_b, P->sfrc,
                                  (double*)P->grid, ks);
        }
        record(P, 3, ks);
        for (auto& B : P->buckets) {
            const PbInst& I0 = P->hinst[B.inst[0]];
            if (mixed)
                launch_kspace_fft<float>(P->d_inst, B.d_inst, (int)B.inst.size(), I0.spec_off, B.M,
                                         (float*)P->grid + I0.grid_off, (float2*)P->spec + I0.spec_off, B.d_tw, ks);
            else
                launch_kspace_fft<double>(P->d_inst, B.d_inst, (int)B.inst.size(), I0.spec_off, B.M,
                                          (double*)P->grid + I0.grid_off, (double2*)P->spec + I0.spec_off, B.d_tw,
                                          ks);
        }
        record(P, 4, ks);
        if (mixed)
            launch_gather<float>(P->d_inst, P->count, P->d_tgt_off, P->n_tgt, P->tpos_a, P->tpos_b,
                                 (const float*)P->grid, (float*)P->u_k, ks);
        else
            launch_gather<double>(P->d_inst, P->count, P->d_tgt_off, P->n_tgt, P->tpos_a, P->tpos_b,
                                  (const double*)P->grid, (double*)P->u_k, ks);
    };
    // The real-space sum and the k-space chain share only the sorted records:
    // the k-space chain runs on a branch forked here and joined before the
    // combine (in the captured graph, two independent branches), so the FFT
    // passes' low occupancy and each kernel's tail are filled by the other
    // branch (N = 1e5 solve 0.866 -> 0.826 ms; the serving stream's large
    // requests 6% faster).  Stage timing keeps the serial order.
    if (P->timing || !P->any_real || !P->any_k) {
        real_part(s);
        record(P, 2, s);
        kspace_part(s);
    } else {
        cudaEventRecord(P->ev_fork, s);
        cudaStreamWaitEvent(P->stream_k, P->ev_fork, 0);
        kspace_part(P->stream_k);
        real_part(s);
        cudaEventRecord(P->ev_join, P->stream_k);
        cudaStreamWaitEvent(s, P->ev_join, 0);
    }
    record(P, 5, s);
    if (P->any_zero) launch_force_sums(P->d_inst, P->f, P->d_src_off, P->count, P->fsum, s);
    if (mixed)
        launch_combine_mixed(P->d_inst, P->count, P->d_tgt_off, P->n_tgt, P->perm_t, P->u_real, (const float*)P->u_k,
                             P->any_real, P->any_k, P->fsum, P->d_tab, P->f, P->d_src_off, P->U, s);
    else
        launch_combine_fp64(P->d_inst, P->count, P->d_tgt_off, P->n_tgt, P->perm_t, P->u_real,
                            (const double*)P->u_k, P->any_real, P->any_k, P->fsum, P->d_tab, P->f, P->d_src_off, P->U,
                            s);
    record(P, 6, s);
}


// Capacity plan: `cfg.max_instances` positions with one FFT grid, capacity
// totals for sources, targets and cells; bound to actual instances by
// pb_plan_bind before each execution (a serving slot).
int build_slot_host(const pb_slot_config* cfg, pb_plan_s* P)
{
    if (!cfg || cfg->max_instances <= 0 || cfg->max_src < 0 || cfg->max_tgt < 0 || cfg->max_cells <= 0)
        return fail(PB_ERR_INVALID, "bad slot configuration");
    for (int a = 0; a < 3; a++)
        if (!is_pow2(cfg->M[a]) || cfg->M[a] < 8 || cfg->M[a] > 1024)
            return fail(PB_ERR_UNSUPPORTED, "slot grid must be powers of two in [8, 1024]");
    if (cfg->precision != PB_PREC_FP64 && cfg->precision != PB_PREC_MIXED) return fail(PB_ERR_INVALID, "bad precision");
    const int B = cfg->max_instances;
    P->count = B;
    P->prec = cfg->precision;
    P->all_same = false;
    P->any_real = P->any_k = P->any_zero = true;
    P->n_src = std::max(cfg->max_src, 1);
    P->n_tgt = std::max(cfg->max_tgt, 1);
    P->n_y = P->n_tgt;
    P->ncell = cfg->max_cells;
    P->npoly = P->npoly_cap = std::max(16, std::min(kMaxPoly, cfg->npoly > 0 ? cfg->npoly : 18));
    P->res.resize(B);
    P->hinst.resize(B);
    P->htab.resize(B);
    P->par.resize(B);
    P->src_off.assign(B + 1, 0);
    P->tgt_off.assign(B + 1, 0);
    P->cell_off.assign(B + 1, 0);
    P->y_off.assign(B + 1, -1);
    Bucket Bk;
    std::memcpy(Bk.M, cfg->M, sizeof(Bk.M));
    size_t gsz = (size_t)Bk.M[0] * Bk.M[1] * Bk.M[2], ssz = (size_t)Bk.M[0] * Bk.M[1] * (Bk.M[2] / 2 + 1);
    P->grid_elems = P->spec_elems = 0;
    // a valid, empty instance for every position
    pb_solve_params d;
    std::memset(&d, 0, sizeof(d));
    d.L[0] = d.L[1] = d.L[2] = 1.0;
    d.alpha = 1.0;
    d.eps = 0.0;
    d.tol = 1e-6;
    d.d = 0.1;
    d.rc = 0.4;
    for (int a = 0; a < 3; a++) d.M[a] = cfg->M[a];
    d.P = 4;
    d.precision = cfg->precision;
    Resolved R;
    int rc = resolve(d, R);
    if (rc) return rc;
    for (int q = 0; q < B; q++) {
        Bk.inst.push_back(q);
        P->hinst[q].grid_off = (long long)P->grid_elems;
        P->hinst[q].spec_off = (long long)P->spec_elems;
        P->hinst[q].bucket = 0;
        P->grid_elems += 4 * gsz;
        P->spec_elems += 3 * ssz;
        P->par[q] = d;
        P->res[q] = R;
        rc = fill_instance(P, q, d, R, 0, 0, 0, P->npoly_cap);
        if (rc) return rc;
        P->hinst[q].ncell = 0;
    }
    P->buckets.push_back(Bk);
    P->bound = 0;
    P->act_src = P->act_tgt = P->act_y = 0;
    return PB_OK;
}

}  // namespace

extern "C" int pb_plan_create_slot(const pb_slot_config* cfg, pb_plan* out)
{
    if (!out) return fail(PB_ERR_INVALID, "bad arguments");
    *out = nullptr;
    if (pb_device_count() <= 0) return fail(PB_ERR_CUDA, "no CUDA device");
    pb_plan_s* P = new pb_plan_s();
    int rc = build_slot_host(cfg, P);
    if (!rc) rc = plan_alloc(P);
    if (rc) {
        plan_free(P);
        return rc;
    }
    *out = P;
    return PB_OK;
}

extern "C" long long pb_slot_estimate_bytes(const pb_slot_config* cfg)
{
    pb_plan_s tmp;
    int rc = build_slot_host(cfg, &tmp);
    if (rc) return rc;
    return (long long)plan_layout(&tmp, false);
}

namespace {

// Binds `count` instances to a capacity plan; tables are built here unless
// prepared ones are given.
int bind_impl(pb_plan P, const pb_solve_params* p, const PbTables* tabs, int count)
{
    if (!P || (count > 0 && !p) || count < 0 || count > P->count) return fail(PB_ERR_INVALID, "bad arguments");
    std::vector<Resolved> R(count);
    std::vector<pb_solve_params> pp(p, p + count);
    long long ns = 0, nt = 0, ny = 0, nc = 0;
    for (int q = 0; q < count; q++) {
        if (pp[q].precision != P->prec) return fail(PB_ERR_INVALID, "instance %d: precision differs from the plan", q);
        const int* Mq = P->hinst[q].M;
        for (int a = 0; a < 3; a++) {
            if (pp[q].M[a] == 0) pp[q].M[a] = Mq[a];
            if (pp[q].M[a] != Mq[a]) return fail(PB_ERR_INVALID, "instance %d: grid differs from position %d", q, q);
        }
        int rc = resolve(pp[q], R[q]);
        if (rc) return rc;
        if (P->all_same && !R[q].same) return fail(PB_ERR_INVALID, "plan holds targets-are-sources instances only");
        ns += R[q].n_src;
        nt += R[q].n_tgt;
        if (!R[q].same) ny += R[q].n_tgt;
        nc += (long long)R[q].nc[0] * R[q].nc[1] * R[q].nc[2];
    }
    if (ns > P->n_src || nt > P->n_tgt || (!P->all_same && ny > P->n_y) || nc > P->ncell)
        return fail(PB_ERR_BUDGET, "bound instances exceed the plan capacity (src %lld/%d, tgt %lld/%d, cells %lld/%d)",
                    ns, P->n_src, nt, P->n_tgt, nc, P->ncell);
    // the previous binding's upload must have left the staging buffer
    cudaError_t e = cudaEventSynchronize(P->ev_upload);
    if (e != cudaSuccess) return fail(PB_ERR_CUDA, "%s", cudaGetErrorString(e));
    int so = 0, to = 0, co = 0, yo = 0;
    for (int q = 0; q < P->count; q++) {
        P->src_off[q] = so;
        P->tgt_off[q] = to;
        P->cell_off[q] = co;
        if (q < count) {
            P->y_off[q] = R[q].same ? -1 : yo;
            if (tabs) {
                set_inst_fields(P->hinst[q], pp[q], R[q], so, to, co);
                P->htab[q] = tabs[q];
            } else {
                int rc = fill_instance(P, q, pp[q], R[q], so, to, co, P->npoly_cap);
                if (rc) return rc;
            }
            P->res[q] = R[q];
            P->par[q] = pp[q];
            so += R[q].n_src;
            to += R[q].n_tgt;
            if (!R[q].same) yo += R[q].n_tgt;
            co += R[q].nc[0] * R[q].nc[1] * R[q].nc[2];
        } else {
            P->y_off[q] = -1;
            PbInst& I = P->hinst[q];
            I.n_src = I.n_tgt = 0;
            I.src_off = so;
            I.tgt_off = to;
            I.cell_off = co;
            I.ncell = 0;
        }
    }
    P->src_off[P->count] = so;
    P->tgt_off[P->count] = to;
    P->cell_off[P->count] = co;
    P->y_off[P->count] = -1;
    assign_splits(P, count);
    char* st = P->staging;
    size_t ot = sizeof(PbInst) * P->count, oo = ot + sizeof(PbTables) * P->count, ob = sizeof(int) * (P->count + 1);
    std::memcpy(st, P->hinst.data(), sizeof(PbInst) * P->count);
    std::memcpy(st + ot, P->htab.data(), sizeof(PbTables) * P->count);
    std::memcpy(st + oo, P->src_off.data(), ob);
    std::memcpy(st + oo + ob, P->tgt_off.data(), ob);
    std::memcpy(st + oo + 2 * ob, P->cell_off.data(), ob);
    std::memcpy(st + oo + 3 * ob, P->y_off.data(), ob);
    P->upload_pending = true;
    P->have_positions = false;
    P->bound = count;
    P->act_src = (int)ns;
    P->act_tgt = (int)nt;
    P->act_y = (int)ny;
    return PB_OK;
}

}  // namespace

extern "C" int pb_plan_bind(pb_plan P, const pb_solve_params* p, int count) { return bind_impl(P, p, nullptr, count); }

namespace pb {

// Uploads a pending binding and runs the device work: eagerly on the first
// execution (and when timing), as a captured CUDA graph afterwards.
int upload_and_compute(pb_plan P, cudaStream_t s, bool forces_only)
{
    if (P->upload_pending) {
        char* st = P->staging;
        size_t oi = 0, ot = oi + sizeof(PbInst) * P->count, oo = ot + sizeof(PbTables) * P->count;
        size_t ob = sizeof(int) * (P->count + 1);
        PB_CK(cudaMemcpyAsync(P->d_inst, st + oi, sizeof(PbInst) * P->count, cudaMemcpyHostToDevice, s));
        PB_CK(cudaMemcpyAsync(P->d_tab, st + ot, sizeof(PbTables) * P->count, cudaMemcpyHostToDevice, s));
        PB_CK(cudaMemcpyAsync(P->d_src_off, st + oo, ob, cudaMemcpyHostToDevice, s));
        PB_CK(cudaMemcpyAsync(P->d_tgt_off, st + oo + ob, ob, cudaMemcpyHostToDevice, s));
        PB_CK(cudaMemcpyAsync(P->d_cell_off, st + oo + 2 * ob, ob, cudaMemcpyHostToDevice, s));
        PB_CK(cudaMemcpyAsync(P->d_y_off, st + oo + 3 * ob, ob, cudaMemcpyHostToDevice, s));
        PB_CK(cudaEventRecord(P->ev_upload, s));
        P->upload_pending = false;
    }
    if (P->n_tgt <= 0 || P->act_tgt <= 0) return PB_OK;
    cudaGraphExec_t& gx = forces_only ? P->gexec_f : P->gexec;
    const int runs = forces_only ? P->fexec_count : P->exec_count;
    if (P->timing || runs < 1) {
        run_compute(P, s, forces_only);
    } else {
        if (!gx) {
            cudaGraph_t g;
            PB_CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            run_compute(P, s, forces_only);
            PB_CK(cudaStreamEndCapture(s, &g));
            if (!forces_only) {
                size_t nn = 0;
                cudaGraphGetNodes(g, nullptr, &nn);
                std::vector<cudaGraphNode_t> nodes(nn);
                cudaGraphGetNodes(g, nodes.data(), &nn);
                P->graph_kernels = 0;
                for (auto nd : nodes) {
                    cudaGraphNodeType ty;
                    if (cudaGraphNodeGetType(nd, &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel)
                        P->graph_kernels++;
                }
            }
            cudaError_t e = cudaGraphInstantiate(&gx, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return fail(PB_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
        }
        PB_CK(cudaGraphLaunch(gx, s));
    }
    PB_CK(cudaGetLastError());
    return PB_OK;
}

int plan_execute_parts(pb_plan P, const double* const* xs, const double* const* fs, const double* const* ys,
                       double* const* Us, cudaStream_t us)
{
    if (!P) return fail(PB_ERR_INVALID, "null plan");
    NvtxRange nv("pb_plan_execute_parts");
    cudaStream_t s = P->stream;
    PB_CK(cudaEventRecord(P->ev_in, us));
    PB_CK(cudaStreamWaitEvent(s, P->ev_in, 0));
    for (int q = 0; q < P->bound; q++) {
        const Resolved& R = P->res[q];
        const size_t so = 3 * (size_t)P->src_off[q];
        if (R.n_src > 0) {
            PB_CK(cudaMemcpyAsync(P->x + so, xs[q], sizeof(double) * 3 * R.n_src, cudaMemcpyHostToDevice, s));
            PB_CK(cudaMemcpyAsync(P->f + so, fs[q], sizeof(double) * 3 * R.n_src, cudaMemcpyHostToDevice, s));
        }
        if (!R.same && R.n_tgt > 0)
            PB_CK(cudaMemcpyAsync(P->y + 3 * (size_t)P->y_off[q], ys[q], sizeof(double) * 3 * R.n_tgt,
                                  cudaMemcpyHostToDevice, s));
    }
    int rc = upload_and_compute(P, s, false);
    if (rc) return rc;
    for (int q = 0; q < P->bound; q++) {
        const Resolved& R = P->res[q];
        if (R.n_tgt > 0)
            PB_CK(cudaMemcpyAsync(Us[q], P->U + 3 * (size_t)P->tgt_off[q], sizeof(double) * 3 * R.n_tgt,
                                  cudaMemcpyDeviceToHost, s));
    }
    PB_CK(cudaMemcpyAsync(P->h_bad, P->d_bad, sizeof(int) * (P->count + 1), cudaMemcpyDeviceToHost, s));
    P->exec_count++;
    PB_CK(cudaEventRecord(P->ev_out, s));
    PB_CK(cudaStreamWaitEvent(us, P->ev_out, 0));
    return PB_OK;
}

int api_error(int code, const char* msg) { return fail(code, "%s", msg); }

namespace {
void fill_info(const Resolved& R, int npoly, pb_instance_info* info)
{
    info->d = R.d;
    info->rc = R.rc;
    info->eta = R.eta;
    info->m_std = R.m;
    for (int a = 0; a < 3; a++) {
        info->M[a] = R.M[a];
        info->ncell[a] = R.nc[a];
    }
    info->P = R.P;
    info->npoly = npoly;
    info->pairs_est = R.pairs_est;
}
}  // namespace

int resolve_info(const pb_solve_params& p, pb_instance_info* info)
{
    Resolved R;
    int rc = resolve(p, R);
    if (rc) return rc;
    fill_info(R, 0, info);
    return PB_OK;
}

int prepare_instance(const pb_solve_params& p, int npoly_cap, PbTables* tab, pb_instance_info* info)
{
    Resolved R;
    int rc = resolve(p, R);
    if (rc) return rc;
    if (build_tables(p.alpha, R.d, p.eps, R.rc, kTableTol, tab, npoly_cap, p.precision == PB_PREC_FP64))
        return fail(PB_ERR_INVALID, "table construction failed");
    fill_info(R, tab->nd, info);
    return PB_OK;
}

int plan_bind_prepared(pb_plan P, const pb_solve_params* p, const PbTables* tabs, int count)
{
    return bind_impl(P, p, tabs, count);
}

const int* plan_bad_flags(pb_plan P) { return P->h_bad; }

int plan_exec_status(pb_plan P) { return P->h_bad[P->count]; }

int kspace_instance(const pb_solve_params& p, PbInst* inst)
{
    Resolved R;
    int rc = resolve(p, R);
    if (rc) return rc;
    std::memset(inst, 0, sizeof(PbInst));
    set_inst_fields(*inst, p, R, 0, 0, 0);
    return PB_OK;
}

}  // namespace pb

extern "C" {

const char* pb_last_error(void) { return g_err.c_str(); }

const char* pb_version(void) { return "periodicbrinkman_gb300 0.1 (sm_103a)"; }

int pb_device_count(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

long long pb_plan_estimate_bytes(const pb_solve_params* p, int count)
{
    if (!p || count <= 0) return fail(PB_ERR_INVALID, "bad arguments");
    pb_plan_s tmp;
    int rc = build_plan_host(p, count, &tmp);
    if (rc) return rc;
    return (long long)plan_layout(&tmp, false);
}

int pb_resolve(const pb_solve_params* p, pb_instance_info* info)
{
    if (!p || !info) return fail(PB_ERR_INVALID, "bad arguments");
    Resolved R;
    int rc = resolve(*p, R);
    if (rc) return rc;
    PbTables T;
    if (build_tables(p->alpha, R.d, p->eps, R.rc, kTableTol, &T, 0, p->precision == PB_PREC_FP64))
        return fail(PB_ERR_INVALID, "table construction failed");
    info->d = R.d;
    info->rc = R.rc;
    info->eta = R.eta;
    info->m_std = R.m;
    for (int a = 0; a < 3; a++) {
        info->M[a] = R.M[a];
        info->ncell[a] = R.nc[a];
    }
    info->P = R.P;
    info->npoly = T.nd;
    info->pairs_est = R.pairs_est;
    return PB_OK;
}

int pb_plan_create(const pb_solve_params* p, int count, pb_plan* out)
{
    if (!p || !out || count <= 0) return fail(PB_ERR_INVALID, "bad arguments");
    *out = nullptr;
    if (pb_device_count() <= 0) return fail(PB_ERR_CUDA, "no CUDA device");
    pb_plan_s* P = new pb_plan_s();
    int rc = build_plan_host(p, count, P);
    if (!rc) rc = plan_alloc(P);
    if (rc) {
        plan_free(P);
        return rc;
    }
    *out = P;
    return PB_OK;
}

int pb_plan_destroy(pb_plan plan)
{
    if (plan) {
        cudaStreamSynchronize(plan->stream);
        plan_free(plan);
    }
    return PB_OK;
}

long long pb_plan_device_bytes(pb_plan plan) { return plan ? (long long)plan->arena_bytes : 0; }

int pb_plan_kernel_count(pb_plan plan) { return plan ? plan->graph_kernels : 0; }

int pb_plan_instance_info(pb_plan plan, int i, pb_instance_info* info)
{
    if (!plan || !info || i < 0 || i >= plan->count) return fail(PB_ERR_INVALID, "bad arguments");
    const Resolved& R = plan->res[i];
    info->d = R.d;
    info->rc = R.rc;
    info->eta = R.eta;
    info->m_std = R.m;
    for (int a = 0; a < 3; a++) {
        info->M[a] = R.M[a];
        info->ncell[a] = R.nc[a];
    }
    info->P = R.P;
    info->npoly = plan->htab[i].nd;
    info->pairs_est = R.pairs_est;
    return PB_OK;
}

int pb_plan_set_timing(pb_plan plan, int enable)
{
    if (!plan) return fail(PB_ERR_INVALID, "null plan");
    plan->timing = enable != 0;
    return PB_OK;
}

int pb_plan_stage_ms(pb_plan plan, double* ms6)
{
    if (!plan || !ms6) return fail(PB_ERR_INVALID, "bad arguments");
    for (int k = 0; k < 6; k++) ms6[k] = plan->stage_ms[k];
    return PB_OK;
}

// Status of the finished last execution from its flags (h_bad).
static int status_of(pb_plan P)
{
    if (P->h_bad[P->count] & kCapItems)
        return fail(PB_ERR_UNSUPPORTED, "real-space work items exceeded the plan's item capacity (%d)", P->item_cap);
    if (P->h_bad[P->count] & kScanStall)
        return fail(PB_ERR_CUDA, "cell-count scan gave up waiting for a preceding block; results not valid");
    for (int q = 0; q < P->count; q++)
        if (P->h_bad[q]) return fail(PB_ERR_INVALID, "non-finite input (instance %d)", q);
    return PB_OK;
}

int pb_plan_status(pb_plan P)
{
    if (!P) return fail(PB_ERR_INVALID, "null plan");
    PB_CK(cudaStreamSynchronize(P->stream));
    return status_of(P);
}

int pb_plan_set_item_capacity(pb_plan P, int cap)
{
    if (!P || cap < 1) return fail(PB_ERR_INVALID, "bad arguments");
    const int full = 4 * std::max(P->n_tgt, 1) + 4096;  // as plan_layout sizes the array
    if (cap > full) return fail(PB_ERR_INVALID, "item capacity above the allocated %d", full);
    PB_CK(cudaStreamSynchronize(P->stream));
    P->item_cap = cap;
    // the captured graphs hold the old capacity in their kernel parameters
    if (P->gexec) cudaGraphExecDestroy(P->gexec);
    if (P->gexec_f) cudaGraphExecDestroy(P->gexec_f);
    P->gexec = P->gexec_f = nullptr;
    P->exec_count = P->fexec_count = 0;
    P->have_positions = false;
    return PB_OK;
}

// One execution of a plan; with `forces_only` the positions (and targets) of
// the last full execution are reused and only `f` is read.
static int execute_impl(pb_plan P, const double* x, const double* f, const double* y, double* U, int where, void* stream_v,
                 bool forces_only)
{
    if (!P) return fail(PB_ERR_INVALID, "null plan");
    NvtxRange nv(forces_only ? "pb_plan_execute_forces" : "pb_plan_execute");
    if (forces_only && !P->have_positions)
        return fail(PB_ERR_INVALID, "no sorted positions: execute the plan with positions first");
    if ((P->act_src > 0 && ((!forces_only && !x) || !f)) || (P->act_tgt > 0 && !U) ||
        (!forces_only && !P->all_same && P->act_y > 0 && !y))
        return fail(PB_ERR_INVALID, "null buffer");
    if (where != PB_HOST && where != PB_DEVICE && where != PB_HOST_PINNED)
        return fail(PB_ERR_INVALID, "bad memory location");
    cudaStream_t us = (cudaStream_t)stream_v;
    cudaStream_t s = P->stream;
    // Non-finite inputs: the asynchronous host path scans them here, before
    // anything is queued; the synchronous host path reads the flags the
    // binning and preparation kernels set (they map such values to finite
    // ones), after the execution, and then fails with U unspecified.
    if (where == PB_HOST_PINNED) {
        for (size_t i = 0; i < 3 * (size_t)P->act_src; i++)
            if ((!forces_only && !std::isfinite(x[i])) || !std::isfinite(f[i]))
                return fail(PB_ERR_INVALID, "non-finite input");
        if (!forces_only && !P->all_same)
            for (size_t i = 0; i < 3 * (size_t)P->act_y; i++)
                if (!std::isfinite(y[i])) return fail(PB_ERR_INVALID, "non-finite target");
    }
    PB_CK(cudaEventRecord(P->ev_in, us));
    PB_CK(cudaStreamWaitEvent(s, P->ev_in, 0));
    cudaMemcpyKind kin = where == PB_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (P->act_src > 0) {
        if (!forces_only) PB_CK(cudaMemcpyAsync(P->x, x, sizeof(double) * 3 * P->act_src, kin, s));
        PB_CK(cudaMemcpyAsync(P->f, f, sizeof(double) * 3 * P->act_src, kin, s));
    }
    if (!forces_only && !P->all_same && P->act_y > 0)
        PB_CK(cudaMemcpyAsync(P->y, y, sizeof(double) * 3 * P->act_y, kin, s));
    // a failed full execution leaves no positions to reuse
    if (!forces_only) P->have_positions = false;
    int rc = upload_and_compute(P, s, forces_only);
    if (rc) return rc;
    if (P->n_tgt > 0 && P->act_tgt > 0) {
        cudaMemcpyKind kout = where == PB_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
        PB_CK(cudaMemcpyAsync(U, P->U, sizeof(double) * 3 * P->act_tgt, kout, s));
    }
    PB_CK(cudaMemcpyAsync(P->h_bad, P->d_bad, sizeof(int) * (P->count + 1), cudaMemcpyDeviceToHost, s));
    if (forces_only)
        P->fexec_count++;
    else
        P->exec_count++;
    PB_CK(cudaEventRecord(P->ev_out, s));
    PB_CK(cudaStreamWaitEvent(us, P->ev_out, 0));
    if (where == PB_HOST || P->timing) PB_CK(cudaStreamSynchronize(s));
    if (where == PB_HOST) {
        int rc = status_of(P);
        if (rc) return rc;
    }
    if (!forces_only) P->have_positions = true;
    if (P->timing) {
        float ms;
        for (int k = 0; k < 6; k++) {
            cudaEventElapsedTime(&ms, P->tev[k], P->tev[k + 1]);
            P->stage_ms[k] = ms;
        }
    }
    return PB_OK;
}

int pb_plan_execute(pb_plan P, const double* x, const double* f, const double* y, double* U, int where,
                    void* stream_v)
{
    return execute_impl(P, x, f, y, U, where, stream_v, false);
}

int pb_plan_execute_forces(pb_plan P, const double* f, double* U, int where, void* stream_v)
{
    return execute_impl(P, nullptr, f, nullptr, U, where, stream_v, true);
}

int pb_solve(const pb_solve_params* p, const double* x, const double* f, const double* y, double* U, int where,
             void* stream)
{
    NvtxRange nv("pb_solve");
    pb_plan P = nullptr;
    int rc = pb_plan_create(p, 1, &P);
    if (rc) return rc;
    rc = pb_plan_execute(P, x, f, y, U, where, stream);
    if (!rc) {
        cudaError_t e = cudaStreamSynchronize(P->stream);
        if (e != cudaSuccess) rc = fail(PB_ERR_CUDA, "%s", cudaGetErrorString(e));
    }
    pb_plan_destroy(P);
    return rc;
}

// ---- reference-facing entry points ----

int pb_periodic_brinkman_ex(double* dA, const double* dx, int m, const double* dx0, int n, double a, double d,
                            double e, const int* Mx, const int* Nx, const double* L, int tau_scaled, void* stream)
{
    if (m < 0 || n < 0 || !L || !Mx || !Nx) return fail(PB_ERR_INVALID, "bad arguments");
    if ((m > 0 && !dx) || (n > 0 && !dx0) || (m > 0 && n > 0 && !dA)) return fail(PB_ERR_INVALID, "null buffer");
    for (int q = 0; q < 3; q++)
        if (!std::isfinite(L[q]) || !(L[q] > 0)) return fail(PB_ERR_INVALID, "L must be > 0");
    if (!std::isfinite(a) || !(a > 0) || !std::isfinite(d) || !(d > 0) || !std::isfinite(e) || e < 0)
        return fail(PB_ERR_INVALID, "need alpha > 0, d > 0, e >= 0");
    if (pb_device_count() <= 0) return fail(PB_ERR_CUDA, "no CUDA device");
    NvtxRange nv("pb_periodic_brinkman");
    int rc = launch_dense_matrix(dA, dx, m, dx0, n, a, d, e, Mx, Nx, L, tau_scaled, (cudaStream_t)stream);
    if (rc) return fail(PB_ERR_UNSUPPORTED, "more than 256 Fourier shells per axis");
    PB_CK(cudaGetLastError());
    return PB_OK;
}

int pb_periodic_brinkman(double* dA, const double* dx, int m, const double* dx0, int n, double a, double d,
                         double e, int M, int N, const double* L, int maxBlockSize)
{
    if (maxBlockSize <= 0) return fail(PB_ERR_INVALID, "maxBlockSize must be > 0");
    if (!L) return fail(PB_ERR_INVALID, "null L");
    // per-axis shell counts (cuda/periodicBrinkman.h:457-487)
    int Mx[3] = {M, M, M}, Nx[3] = {N, N, N}, idL[3] = {0, 1, 2}, t;
    if (L[idL[0]] > L[idL[1]]) {
        t = idL[0];
        idL[0] = idL[1];
        idL[1] = t;
    }
    if (L[idL[2]] <= L[idL[0]]) {
        t = idL[2];
        idL[2] = idL[1];
        idL[1] = idL[0];
        idL[0] = t;
    } else if (L[idL[2]] < L[idL[1]]) {
        t = idL[1];
        idL[1] = idL[2];
        idL[2] = t;
    }
    Mx[idL[2]] = (int)std::ceil(M * L[idL[0]] / L[idL[2]]);
    Mx[idL[1]] = (int)std::ceil(M * L[idL[0]] / L[idL[1]]);
    Nx[idL[0]] = (int)std::ceil(N * L[idL[2]] / L[idL[0]]);
    Nx[idL[1]] = (int)std::ceil(N * L[idL[2]] / L[idL[1]]);
    if (M < 0) Mx[0] = Mx[1] = Mx[2] = -1;
    if (N <= 0) Nx[0] = Nx[1] = Nx[2] = 0;
    int rc = pb_periodic_brinkman_ex(dA, dx, m, dx0, n, a, d, e, Mx, Nx, L, 1, nullptr);
    if (rc) return rc;
    PB_CK(cudaStreamSynchronize(nullptr));
    return PB_OK;
}

int pb_fft_brinkman(double* U, const double* y, int m_tgt, const double* f, const double* xn, int n,
                    const double* L, const int* M, const int* P, int msd, int C, double e, double tol, double d,
                    double alpha)
{
    (void)C;
    (void)tol;
    if (!L || !M || !P || msd <= 0) return fail(PB_ERR_INVALID, "bad arguments");
    pb_solve_params p;
    std::memset(&p, 0, sizeof(p));
    p.n_src = n;
    p.n_tgt = m_tgt;
    if (m_tgt == 0) return PB_OK;
    for (int a = 0; a < 3; a++) {
        p.L[a] = L[a];
        p.M[a] = M[a];
    }
    p.alpha = alpha;
    p.eps = e;
    p.d = d;
    p.P = P[0];
    p.m_std = msd;
    p.tol = 1e-6;
    p.rc = d;  // unused: k space only
    p.precision = PB_PREC_FP64;
    p.flags = PB_KSPACE;
    return pb_solve(&p, xn, f, y, U, PB_HOST, nullptr);
}

int pb_debug_pair_kernel64(double alpha, double d, double eps, double rc, int n, const double* r, double* H1,
                           double* H2)
{
    PbTables T;
    if (build_tables(alpha, d, eps, rc, kTableTol, &T, 0, true)) return fail(PB_ERR_INVALID, "bad kernel parameters");
    for (int i = 0; i < n; i++) {
        const double ri = r[i], r2 = ri * ri;
        if (r2 < T.rtiny2 || r2 == 0.0) {  // the FP64 small-r series (eps > 0) or the r -> 0 limit
            double s1 = 0, s2 = 0;
            if (T.blob) {
                s1 = T.ser1[kNumSeries - 1];
                s2 = T.ser2[kNumSeries - 1];
                for (int m = kNumSeries - 2; m >= 0; m--) {
                    s1 = std::fma(s1, r2, T.ser1[m]);
                    s2 = std::fma(s2, r2, T.ser2[m]);
                }
            } else {
                s1 = T.self1;
            }
            H1[i] = s1;
            H2[i] = s2;
        } else if (T.nf > 0 && r2 >= T.rf2) {  // the FP64 far series, by the GPU's Clenshaw recurrence
            const double t = std::fma(ri, T.tf_scale, T.tf_off), t2 = 2.0 * t;
            double b1x = 0, b1y = 0, b2x = 0, b2y = 0;
            for (int k = T.nf - 1; k >= 1; k--) {
                const double b0x = std::fma(t2, b1x, T.cf1[k] - b2x), b0y = std::fma(t2, b1y, T.cf2[k] - b2y);
                b2x = b1x;
                b1x = b0x;
                b2y = b1y;
                b1y = b0y;
            }
            H1[i] = std::fma(t, b1x, T.cf1[0] - b2x) / ri;
            H2[i] = std::fma(t, b1y, T.cf2[0] - b2y) / (r2 * ri);
        } else {  // the closed forms, as the GPU's FP64 kernel evaluates them there
            double h1 = 0, h2 = 0;
            diffH_closed(ri, alpha, d, &h1, &h2);
            if (T.blob && r2 < (double)T.rs2) {
                double e1, e2;
                diffH_closed(ri, alpha, eps, &e1, &e2);
                h1 -= e1;
                h2 -= e2;
            }
            H1[i] = h1;
            H2[i] = h2;
        }
    }
    return PB_OK;
}

int pb_debug_fft_green(const pb_solve_params* p, void* grid, void* stream)
{
    if (!p || !grid) return fail(PB_ERR_INVALID, "bad arguments");
    for (int a = 0; a < 3; a++)
        if (p->M[a] <= 0) return fail(PB_ERR_INVALID, "the grid M must be given");
    Resolved R;
    int rc = resolve(*p, R);
    if (rc) return rc;
    if (pb_device_count() <= 0) return fail(PB_ERR_CUDA, "no CUDA device");
    PbInst I;
    std::memset(&I, 0, sizeof(I));
    set_inst_fields(I, *p, R, 0, 0, 0);
    I.n_src = I.n_tgt = 1;  // a live instance for the passes
    const bool fp64 = p->precision == PB_PREC_FP64;
    const size_t esz = fp64 ? 8 : 4, spec = 3 * (size_t)R.M[0] * R.M[1] * (R.M[2] / 2 + 1) * 2 * esz;
    const size_t twb = twiddle_bytes(R.M, fp64);
    std::vector<char> tw(twb);
    fill_twiddles(R.M, fp64, tw.data());
    const size_t o_inst = 0, o_b = align_up(sizeof(PbInst)), o_tw = o_b + 256, o_spec = o_tw + align_up(twb);
    char* arena = nullptr;
    cudaError_t e = cudaMalloc(&arena, o_spec + spec);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(PB_ERR_NOMEM, "device allocation failed");
    }
    cudaStream_t s = (cudaStream_t)stream;
    const int zero = 0;
    e = cudaMemcpy(arena + o_inst, &I, sizeof(I), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(arena + o_b, &zero, sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(arena + o_tw, tw.data(), twb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        if (fp64)
            launch_kspace_fft<double>((const PbInst*)(arena + o_inst), (const int*)(arena + o_b), 1, 0, R.M,
                                      (double*)grid, arena + o_spec, arena + o_tw, s);
        else
            launch_kspace_fft<float>((const PbInst*)(arena + o_inst), (const int*)(arena + o_b), 1, 0, R.M,
                                     (float*)grid, arena + o_spec, arena + o_tw, s);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(arena);
    if (e != cudaSuccess) return fail(PB_ERR_CUDA, "%s", cudaGetErrorString(e));
    return PB_OK;
}

int pb_debug_pair_kernel(double alpha, double d, double eps, double rc, int n, const double* r, double* H1,
                         double* H2)
{
    PbTables T;
    if (build_tables(alpha, d, eps, rc, kTableTol, &T)) return fail(PB_ERR_INVALID, "bad kernel parameters");
    for (int i = 0; i < n; i++) {
        float rf = (float)r[i];
        float r2 = rf * rf;
        if (r2 < T.rtiny2f || r2 == 0.f) {
            double rr = (double)rf * rf, h1 = 0, h2 = 0;
            if (T.blob) {
                double p1 = T.ser1[kNumSeries - 1], p2 = T.ser2[kNumSeries - 1];
                for (int m = kNumSeries - 2; m >= 0; m--) {
                    p1 = p1 * rr + T.ser1[m];
                    p2 = p2 * rr + T.ser2[m];
                }
                h1 = p1;
                h2 = p2;
            } else {
                h1 = T.self1;
            }
            H1[i] = h1;
            H2[i] = h2;
            continue;
        }
        float ri = 1.0f / rf;
        auto poly = [&](const float* c1, const float* c2, int n, float t, float& p1, float& p2) {
            p1 = c1[n - 1];
            p2 = c2[n - 1];
            for (int k = n - 2; k >= 0; k--) {
                p1 = std::fma(p1, t, c1[k]);
                p2 = std::fma(p2, t, c2[k]);
            }
        };
        auto cheb = [&](const float* c1, const float* c2, int n, float t, float& p1, float& p2) {
            float a1 = 0, a2 = 0, b1 = 0, b2 = 0;  // Clenshaw, as the kernel does
            for (int k = n - 1; k >= 1; k--) {
                float n1 = std::fma(2.f * t, a1, c1[k] - b1), n2 = std::fma(2.f * t, a2, c2[k] - b2);
                b1 = a1;
                b2 = a2;
                a1 = n1;
                a2 = n2;
            }
            p1 = std::fma(t, a1, c1[0] - b1);
            p2 = std::fma(t, a2, c2[0] - b2);
        };
        float T1, T2;
        if (r2 < T.rs2) {  // blob piece: H itself
            float h1, h2;
            cheb(T.cb1, T.cb2, T.nb, std::fma(rf, T.tb_scale, T.tb_off), h1, h2);
            H1[i] = h1;
            H2[i] = h2 * (ri * ri);
            continue;
        }
        if (r2 < T.rm2)
            cheb(T.cn1, T.cn2, T.nn, std::fma(rf, T.tn_scale, T.tn_off), T1, T2);
        else
            poly(T.pd1, T.pd2, T.nd, std::fma(rf, T.td_scale, T.td_off), T1, T2);
        H1[i] = T1 * ri;
        H2[i] = T2 * (ri * ri * ri);
    }
    return PB_OK;
}

}  // extern "C"

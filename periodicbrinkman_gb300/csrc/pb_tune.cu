// Tuning report: measured error against the splitting parameters, the study
// the reference runs by hand (its driver computes the direct-Ewald matrix for
// eight splitting widths and records max|A(d) - A(d0)|, cuda/periodicBrinkman.cu
// :139-203; its commented-out optimalNumShells grows the shells until an
// error target is met, cuda/periodicBrinkman.h:836-1015).  The Ewald total
// does not depend on the splitting width d, so every candidate's velocities
// are compared with one reference solution of the same instance: the FP64
// path at a tight tolerance, autotuned.  Each row reports the parameters the
// candidate resolved to (d, rc, grid, support), its max and RMS relative
// error and its device time.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "pb_internal.h"
#include "pbrinkman.h"

using namespace pb;

namespace {

void rel_errors(const std::vector<double>& u, const std::vector<double>& r, double* mx, double* rms)
{
    double nmax = 0, dmax = 0, s_d = 0, s_r = 0;
    for (size_t i = 0; i + 2 < r.size(); i += 3) {
        double dd = 0, rr = 0;
        for (int c = 0; c < 3; c++) {
            const double e = u[i + c] - r[i + c];
            dd += e * e;
            rr += r[i + c] * r[i + c];
        }
        nmax = std::max(nmax, rr);
        dmax = std::max(dmax, dd);
        s_d += dd;
        s_r += rr;
    }
    *mx = nmax > 0 ? std::sqrt(dmax / nmax) : std::sqrt(dmax);
    *rms = s_r > 0 ? std::sqrt(s_d / s_r) : std::sqrt(s_d);
}

struct Buffers {
    char* base = nullptr;
    ~Buffers()
    {
        if (base) cudaFree(base);
    }
};

}  // namespace

extern "C" int pb_tune_report(const pb_solve_params* p, const double* x, const double* f, const double* y, int where,
                              const double* d_values, int nd, double ref_tol, pb_tune_row* rows)
{
    NvtxRange nv("pb_tune_report");
    if (!p || nd < 0 || (nd > 0 && (!d_values || !rows)) || (where != PB_HOST && where != PB_DEVICE))
        return api_error(PB_ERR_INVALID, "bad arguments");
    if (!(ref_tol >= 0) || ref_tol >= 1e-3) return api_error(PB_ERR_INVALID, "ref_tol must be in [0, 1e-3)");
    for (int k = 0; k < nd; k++)
        if (!std::isfinite(d_values[k]) || d_values[k] < 0) return api_error(PB_ERR_INVALID, "d values must be >= 0");
    pb_instance_info info;
    int rc = resolve_info(*p, &info);
    if (rc) return rc;
    const int n = p->n_src, m = p->n_tgt > 0 ? p->n_tgt : p->n_src;
    if (m <= 0) return PB_OK;
    if (!x || !f || (p->n_tgt > 0 && !y)) return api_error(PB_ERR_INVALID, "null buffer");
    if (pb_device_count() <= 0) return api_error(PB_ERR_CUDA, "no CUDA device");
    // device copies of the inputs (host callers), the reference and one candidate's velocities
    const size_t bx = 3 * (size_t)std::max(n, 1) * sizeof(double), by = 3 * (size_t)m * sizeof(double);
    Buffers B;
    if (cudaMalloc(&B.base, 2 * bx + 3 * by) != cudaSuccess) {
        cudaGetLastError();
        return api_error(PB_ERR_NOMEM, "device allocation failed");
    }
    double *dx = (double*)B.base, *df = (double*)(B.base + bx), *dy = (double*)(B.base + 2 * bx);
    double *dref = (double*)(B.base + 2 * bx + by), *du = (double*)(B.base + 2 * bx + 2 * by);
    const cudaMemcpyKind kin = where == PB_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    cudaError_t e = cudaMemcpy(dx, x, 3 * (size_t)n * sizeof(double), kin);
    if (e == cudaSuccess) e = cudaMemcpy(df, f, 3 * (size_t)n * sizeof(double), kin);
    if (e == cudaSuccess && p->n_tgt > 0) e = cudaMemcpy(dy, y, by, kin);
    if (e != cudaSuccess) return api_error(PB_ERR_CUDA, cudaGetErrorString(e));
    const double* ytgt = p->n_tgt > 0 ? dy : nullptr;
    // the reference solution: FP64, tight tolerance, every tuning field autotuned
    pb_solve_params pr = *p;
    pr.precision = PB_PREC_FP64;
    pr.tol = ref_tol > 0 ? ref_tol : 1e-12;
    pr.d = pr.rc = pr.m_std = 0;
    pr.P = 0;
    pr.M[0] = pr.M[1] = pr.M[2] = 0;
    rc = pb_solve(&pr, dx, df, ytgt, dref, PB_DEVICE, nullptr);
    if (rc) return rc;
    std::vector<double> uref(3 * (size_t)m), u(3 * (size_t)m);
    if ((e = cudaMemcpy(uref.data(), dref, by, cudaMemcpyDeviceToHost)) != cudaSuccess)
        return api_error(PB_ERR_CUDA, cudaGetErrorString(e));
    cudaStream_t s = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&ev[0]) != cudaSuccess ||
        cudaEventCreate(&ev[1]) != cudaSuccess)
        return api_error(PB_ERR_CUDA, "stream or event creation failed");
    for (int k = 0; k < nd; k++) {
        pb_tune_row& R = rows[k];
        std::memset(&R, 0, sizeof(R));
        pb_solve_params pk = *p;
        pk.d = d_values[k];
        if (pk.d > 0) pk.rc = p->rc;  // rc = 0: autotuned for this d
        pb_plan plan = nullptr;
        R.status = pb_plan_create(&pk, 1, &plan);
        if (R.status == PB_OK) {
            pb_instance_info ik;
            pb_plan_instance_info(plan, 0, &ik);
            R.d = ik.d;
            R.rc = ik.rc;
            for (int a = 0; a < 3; a++) R.M[a] = ik.M[a];
            R.P = ik.P;
            R.pairs_est = ik.pairs_est;
            // eager, captured, then three timed replays (median)
            for (int w = 0; w < 2 && R.status == PB_OK; w++) R.status = pb_plan_execute(plan, dx, df, ytgt, du, PB_DEVICE, s);
            float t3[3] = {0, 0, 0};
            for (int r = 0; r < 3 && R.status == PB_OK; r++) {
                cudaEventRecord(ev[0], s);
                R.status = pb_plan_execute(plan, dx, df, ytgt, du, PB_DEVICE, s);
                cudaEventRecord(ev[1], s);
                if (cudaEventSynchronize(ev[1]) != cudaSuccess) R.status = PB_ERR_CUDA;
                cudaEventElapsedTime(&t3[r], ev[0], ev[1]);
            }
            if (R.status == PB_OK) R.status = pb_plan_status(plan);
            std::sort(t3, t3 + 3);
            R.ms = t3[1];
            if (R.status == PB_OK && cudaMemcpy(u.data(), du, by, cudaMemcpyDeviceToHost) != cudaSuccess)
                R.status = PB_ERR_CUDA;
            if (R.status == PB_OK) rel_errors(u, uref, &R.max_err, &R.rms_err);
        }
        if (plan) pb_plan_destroy(plan);
        if (R.status != PB_OK) R.max_err = R.rms_err = -1;
    }
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    cudaStreamDestroy(s);
    return PB_OK;
}

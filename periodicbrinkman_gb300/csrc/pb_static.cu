// Allocation-free k-space evaluation: the velocities of pb_fft_brinkman with
// every intermediate buffer in one fixed array compiled into the library's
// device image, for callers that must not allocate device memory (cudaMalloc
// and cudaFree can block or synchronise the whole device, and some host
// programs own all device memory through their own pool).  Device pointers in
// and out, one stream, no cudaMalloc/cudaFree and no allocating library call.
//
// Limits: grid <= 64 points per axis, <= 65536 sources and <= 65536 targets.
// The array (21.2 MB) is held by every GPU that loads the library until
// the process exits.  Every call shares it and it keeps the last call's
// contents, so the grid is cleared at the start of each call, and calls that
// overlap on the GPU (other streams, other host threads) race.
//
// The instance descriptor and the FFT twiddles are built on the host and
// handed to a one-block set-up kernel as its (by-value) launch parameter,
// which writes them into the array: no host-to-device copy from pageable
// memory, which the driver could stage through its own buffer and order
// against the whole device.
#include <cstring>
#include <mutex>

#include "pb_device.cuh"
#include "pb_internal.h"
#include "pb_kernels.h"

using namespace pb;

namespace {

constexpr int kStaticMaxGrid = 64;
constexpr int kStaticMaxPoints = 65536;
constexpr int kStaticMaxDevices = 64;

constexpr size_t al256(size_t v) { return (v + 255) & ~(size_t)255; }

// The instance descriptor and the offset arrays the kernels read, staged
// from the host in one copy.
struct StaticHeader {
    PbInst inst;
    int src_off[2];
    int tgt_off[2];
    int bucket[1];
};

constexpr size_t kGridMax = (size_t)kStaticMaxGrid * kStaticMaxGrid * kStaticMaxGrid;
constexpr size_t kOffHeader = 0;
constexpr size_t kOffTw = kOffHeader + al256(sizeof(StaticHeader));
constexpr size_t kTwMax = 4096;  // twiddles of a 64^3 grid: 113 double2
constexpr size_t kOffSpos = kOffTw + kTwMax;
constexpr size_t kOffSfrc = kOffSpos + al256(kStaticMaxPoints * sizeof(Dbl4));
constexpr size_t kOffTpos = kOffSfrc + al256(kStaticMaxPoints * sizeof(Dbl4));
constexpr size_t kOffGrid = kOffTpos + al256(kStaticMaxPoints * sizeof(Dbl4));
constexpr size_t kOffSpec = kOffGrid + al256(4 * kGridMax * sizeof(double));  // 4 planes per instance
constexpr size_t kScratchBytes =
    kOffSpec + al256(3 * (size_t)kStaticMaxGrid * kStaticMaxGrid * (kStaticMaxGrid / 2 + 1) * sizeof(double2));

// Launch parameter of the set-up kernel: the header and the twiddle table
// (4.6 KB, within the 32 KB a kernel parameter list may hold on this GPU).
struct StaticSetup {
    StaticHeader h;
    alignas(16) unsigned char tw[kTwMax];
};
static_assert(sizeof(StaticHeader) % 4 == 0 && kTwMax % 4 == 0, "word copies");
static_assert(sizeof(StaticSetup) < 30000, "kernel parameter size");

}  // namespace

// The scratch array.  In host code this name is only a stand-in for the
// symbol: its device address comes from cudaGetSymbolAddress, per device.
static __device__ __align__(256) unsigned char g_static_scratch[kScratchBytes];

namespace {

std::mutex g_static_mu;
void* g_static_ptr[kStaticMaxDevices] = {};

// Device address of the scratch array on the current device (resolved once
// per device, with that device current).
int static_scratch(char** out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return api_error(PB_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kStaticMaxDevices) return api_error(PB_ERR_UNSUPPORTED, "device index beyond 63");
    std::lock_guard<std::mutex> lk(g_static_mu);
    if (!g_static_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return api_error(PB_ERR_CUDA, "cudaGetSymbolAddress of the static scratch array failed");
        }
        g_static_ptr[dev] = p;
    }
    *out = (char*)g_static_ptr[dev];
    return PB_OK;
}

// Writes the header and `twn` bytes of twiddles from the launch parameter
// into the scratch array (one block).
__global__ void k_static_setup(const StaticSetup su, unsigned* __restrict__ hdr, unsigned* __restrict__ tw, int twn)
{
    const unsigned* hs = reinterpret_cast<const unsigned*>(&su.h);
    const unsigned* ts = reinterpret_cast<const unsigned*>(su.tw);
    for (int i = threadIdx.x; i < (int)(sizeof(StaticHeader) / 4); i += blockDim.x) hdr[i] = hs[i];
    for (int i = threadIdx.x; i < twn / 4; i += blockDim.x) tw[i] = ts[i];
}

// Positions wrapped into the box as FP64 records of instance 0, forces beside.
__global__ void k_static_records(const double* __restrict__ pos, const double* __restrict__ frc, int n, double L0,
                                 double L1, double L2, Dbl4* __restrict__ pos_out, Dbl4* __restrict__ frc_out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* p = pos + 3 * (size_t)i;
    pos_out[i] = make_dbl4(wrap_coord(p[0], L0), wrap_coord(p[1], L1), wrap_coord(p[2], L2), 0.0);
    if (frc) frc_out[i] = make_dbl4(frc[3 * (size_t)i], frc[3 * (size_t)i + 1], frc[3 * (size_t)i + 2], 0.0);
}

}  // namespace

extern "C" int pb_fft_brinkman_static(double* U, const double* y, int m_tgt, const double* f, const double* xn,
                                      int n, const double* L, const int* M, const int* P, int msd, double e, double d,
                                      double alpha, void* stream)
{
    if (!L || !M || !P || msd <= 0 || n < 0 || m_tgt < 0) return api_error(PB_ERR_INVALID, "bad arguments");
    if (m_tgt == 0) return PB_OK;
    if (!U || !y || (n > 0 && (!f || !xn))) return api_error(PB_ERR_INVALID, "bad arguments: null buffer");
    if (n > kStaticMaxPoints || m_tgt > kStaticMaxPoints)
        return api_error(PB_ERR_UNSUPPORTED,
                         "pb_fft_brinkman_static: more than 65536 sources or targets exceeds its static scratch");
    // the grid is the caller's (no autotuning here: an autotuned grid could
    // outgrow the array) and the support must be given
    for (int a = 0; a < 3; a++)
        if (M[a] <= 0) return api_error(PB_ERR_INVALID, "pb_fft_brinkman_static: M[a] must be given (> 0)");
    for (int a = 0; a < 3; a++)
        if (M[a] > kStaticMaxGrid)
            return api_error(PB_ERR_UNSUPPORTED,
                             "pb_fft_brinkman_static: grid above 64 points per axis exceeds its static scratch");
    if (P[0] <= 0) return api_error(PB_ERR_INVALID, "pb_fft_brinkman_static: support P[0] must be > 0");
    // the parameter mapping of pb_fft_brinkman (k space only, FP64)
    pb_solve_params p;
    std::memset(&p, 0, sizeof(p));
    p.n_src = n;
    p.n_tgt = m_tgt;
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
    p.rc = d;
    p.precision = PB_PREC_FP64;
    p.flags = PB_KSPACE;
    StaticSetup su;
    std::memset(&su, 0, sizeof(su));
    StaticHeader& h = su.h;
    int rc = kspace_instance(p, &h.inst);
    if (rc) return rc;
    // every kernel below indexes the grid the descriptor holds: it must be the
    // caller's, within the array, with the support inside it
    for (int a = 0; a < 3; a++)
        if (h.inst.M[a] != M[a] || h.inst.M[a] > kStaticMaxGrid || h.inst.Pa[a] <= 0 || h.inst.Pa[a] > h.inst.M[a])
            return api_error(PB_ERR_UNSUPPORTED, "pb_fft_brinkman_static: grid or support outside its static scratch");
    h.src_off[1] = n;
    h.tgt_off[1] = m_tgt;
    const int Mi[3] = {h.inst.M[0], h.inst.M[1], h.inst.M[2]};
    const size_t twn = twiddle_bytes(Mi, true);
    if (twn > kTwMax || twn % 4) return api_error(PB_ERR_UNSUPPORTED, "twiddle table exceeds its slot");
    fill_twiddles(Mi, true, su.tw);
    char* base = nullptr;
    rc = static_scratch(&base);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    StaticHeader* dh = (StaticHeader*)(base + kOffHeader);
    Dbl4* spos = (Dbl4*)(base + kOffSpos);
    Dbl4* sfrc = (Dbl4*)(base + kOffSfrc);
    Dbl4* tpos = (Dbl4*)(base + kOffTpos);
    double* grid = (double*)(base + kOffGrid);
    double2* spec = (double2*)(base + kOffSpec);
    k_static_setup<<<1, 256, 0, s>>>(su, (unsigned*)dh, (unsigned*)(base + kOffTw), (int)twn);
    cudaError_t ce = cudaGetLastError();
    if (ce == cudaSuccess) ce = cudaMemsetAsync(grid, 0, 4 * (size_t)Mi[0] * Mi[1] * Mi[2] * sizeof(double), s);
    if (ce != cudaSuccess) return api_error(PB_ERR_CUDA, cudaGetErrorString(ce));
    if (n > 0)
        k_static_records<<<(n + 255) / 256, 256, 0, s>>>(xn, f, n, L[0], L[1], L[2], spos, sfrc);
    k_static_records<<<(m_tgt + 255) / 256, 256, 0, s>>>(y, nullptr, m_tgt, L[0], L[1], L[2], tpos, nullptr);
    launch_spread<double>(&dh->inst, 1, dh->src_off, n, spos, nullptr, sfrc, grid, s);
    launch_kspace_fft<double>(&dh->inst, dh->bucket, 1, 0, Mi, grid, spec, base + kOffTw, s);
    launch_gather<double>(&dh->inst, 1, dh->tgt_off, m_tgt, tpos, nullptr, grid, U, s);
    ce = cudaGetLastError();
    if (ce != cudaSuccess) return api_error(PB_ERR_CUDA, cudaGetErrorString(ce));
    return PB_OK;
}

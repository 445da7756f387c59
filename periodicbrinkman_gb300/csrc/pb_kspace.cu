// k-space Ewald sum by spectral Ewald: Gaussian spreading of the three force
// components onto an M^3 grid, batched 3D real FFT, multiplication by the
// screened Brinkman Green tensor with Gaussian deconvolution, inverse FFT and
// Gaussian gather (the algorithm of cuda/fftBrinkman.h:101-273, with a
// centred support window, no spectrum conjugation and per-target support
// gather).  Also the final FP64 combine of real space, k space, self and the
// optional k = 0 mode.
//
// FFT: hand-written shared-memory Stockham radix-2 passes along z (real-to-
// complex by the packed half-length transform), y, and x; the x pass of the
// forward transform is fused with the Green multiplication and the x pass of
// the inverse, so the spectrum is read and written once for all three.
#include "pb_device.cuh"
#include "pb_kernels.h"

namespace pb {

template <class T>
struct Cx;
template <>
struct Cx<float> {
    typedef float2 t;
};
template <>
struct Cx<double> {
    typedef double2 t;
};

template <class T2>
__device__ __forceinline__ T2 cmul(T2 a, T2 b)
{
    T2 r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}

// ---------------------------------------------------------------------------
// Spreading and gathering
// ---------------------------------------------------------------------------

// Sorted positions: mixed (float4 hi, float4 lo, instance in hi.w bits) or FP64 (Dbl4, instance in w).
__device__ __forceinline__ void load_pos(const float4* a, const float4* b, int i, double* x, int& q)
{
    float4 h = a[i], l = b[i];
    x[0] = (double)h.x + (double)l.x;
    x[1] = (double)h.y + (double)l.y;
    x[2] = (double)h.z + (double)l.z;
    q = __float_as_int(h.w);
}
__device__ __forceinline__ void load_pos(const Dbl4* a, const Dbl4* /*b*/, int i, double* x, int& q)
{
    Dbl4 h = a[i];
    x[0] = h.x;
    x[1] = h.y;
    x[2] = h.z;
    q = (int)h.w;
}
__device__ __forceinline__ void load_frc(const float4* f, int i, double* v)
{
    float4 h = f[i];
    v[0] = h.x;
    v[1] = h.y;
    v[2] = h.z;
}
__device__ __forceinline__ void load_frc(const Dbl4* f, int i, double* v)
{
    Dbl4 h = f[i];
    v[0] = h.x;
    v[1] = h.y;
    v[2] = h.z;
}

constexpr int kSpreadWarps = 8;
constexpr int kMaxP = 32;

// Per-axis Gaussian weights exp(-(x - (g0+p) h)^2 / eta) and wrapped grid
// indices of the P-point window centred on x (lane p computes entry p).
template <class T>
__device__ __forceinline__ void window(const PbInst& I, const double* x, int lane, T (*wgt)[kMaxP],
                                       int (*idx)[kMaxP])
{
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int P = I.Pa[a];
        if (lane < P) {
            double h = I.gh[a];
            int g0 = (int)floor(x[a] / h) - P / 2 + 1;
            double base = x[a] - (double)g0 * h;
            T dx = (T)(base - (double)lane * h);
            wgt[a][lane] = exp(-dx * dx / (T)I.eta);
            int g = (g0 + lane) % I.M[a];
            idx[a][lane] = g < 0 ? g + I.M[a] : g;
        }
    }
}

template <class T, class PV, class FV>
__global__ void __launch_bounds__(kSpreadWarps * 32)
    k_spread(const PbInst* __restrict__ inst, const int* __restrict__ ntot_p, const PV* __restrict__ pa,
             const PV* __restrict__ pb, const FV* __restrict__ frc, T* __restrict__ grid)
{
    const int ntot = *ntot_p;
    __shared__ T wgt[kSpreadWarps][3][kMaxP];
    __shared__ int gidx[kSpreadWarps][3][kMaxP];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int s = blockIdx.x * kSpreadWarps + w;
    if (s >= ntot) return;
    double x[3], fv[3];
    int q;
    load_pos(pa, pb, s, x, q);
    load_frc(frc, s, fv);
    const PbInst& I = inst[q];
    window<T>(I, x, lane, wgt[w], gidx[w]);
    __syncwarp();
    const int Py = I.Pa[1], Pz = I.Pa[2], P2 = Py * Pz, P3 = I.Pa[0] * P2;
    const size_t comp = (size_t)I.M[0] * I.M[1] * I.M[2];
    T* g0 = grid + I.grid_off;
    const T f0 = (T)fv[0], f1 = (T)fv[1], f2 = (T)fv[2];
    for (int id = lane; id < P3; id += 32) {
        int px = id / P2, r = id - px * P2, py = r / Pz, pz = r - py * Pz;
        T wv = wgt[w][0][px] * wgt[w][1][py] * wgt[w][2][pz];
        size_t o = ((size_t)gidx[w][0][px] * I.M[1] + gidx[w][1][py]) * I.M[2] + gidx[w][2][pz];
        atomicAdd(g0 + o, f0 * wv);
        atomicAdd(g0 + comp + o, f1 * wv);
        atomicAdd(g0 + 2 * comp + o, f2 * wv);
    }
}

template <class T, class PV>
__global__ void __launch_bounds__(kSpreadWarps * 32)
    k_gather(const PbInst* __restrict__ inst, const int* __restrict__ ntot_p, const PV* __restrict__ pa,
             const PV* __restrict__ pb, const T* __restrict__ grid, T* __restrict__ u_k)
{
    const int ntot = *ntot_p;
    __shared__ T wgt[kSpreadWarps][3][kMaxP];
    __shared__ int gidx[kSpreadWarps][3][kMaxP];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int s = blockIdx.x * kSpreadWarps + w;
    if (s >= ntot) return;
    double x[3];
    int q;
    load_pos(pa, pb, s, x, q);
    const PbInst& I = inst[q];
    window<T>(I, x, lane, wgt[w], gidx[w]);
    __syncwarp();
    const int Py = I.Pa[1], Pz = I.Pa[2], P2 = Py * Pz, P3 = I.Pa[0] * P2;
    const size_t comp = (size_t)I.M[0] * I.M[1] * I.M[2];
    const T* g0 = grid + I.grid_off;
    T s0 = 0, s1 = 0, s2 = 0, c0 = 0, c1 = 0, c2 = 0;
    for (int id = lane; id < P3; id += 32) {
        int px = id / P2, r = id - px * P2, py = r / Pz, pz = r - py * Pz;
        T wv = wgt[w][0][px] * wgt[w][1][py] * wgt[w][2][pz];
        size_t o = ((size_t)gidx[w][0][px] * I.M[1] + gidx[w][1][py]) * I.M[2] + gidx[w][2][pz];
        T v0 = wv * __ldg(g0 + o), v1 = wv * __ldg(g0 + comp + o), v2 = wv * __ldg(g0 + 2 * comp + o);
        // Kahan: running value s - c
        T y = v0 - c0, t = s0 + y;
        c0 = (t - s0) - y;
        s0 = t;
        y = v1 - c1;
        t = s1 + y;
        c1 = (t - s1) - y;
        s1 = t;
        y = v2 - c2;
        t = s2 + y;
        c2 = (t - s2) - y;
        s2 = t;
    }
    s0 -= c0;
    s1 -= c1;
    s2 -= c2;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(kFull, s0, o);
        s1 += __shfl_xor_sync(kFull, s1, o);
        s2 += __shfl_xor_sync(kFull, s2, o);
    }
    if (lane == 0) {
        u_k[3 * (size_t)s] = s0;
        u_k[3 * (size_t)s + 1] = s1;
        u_k[3 * (size_t)s + 2] = s2;
    }
}

template <class T>
void launch_spread(const PbInst* inst, int ninst, const int* src_offsets, int ncap, const void* pos_a,
                   const void* pos_b, const void* frc, T* grid, cudaStream_t s)
{
    if (ncap <= 0) return;
    int blocks = (ncap + kSpreadWarps - 1) / kSpreadWarps;
    const int* ntot = src_offsets + ninst;
    if (sizeof(T) == 4)
        k_spread<T, float4, float4><<<blocks, kSpreadWarps * 32, 0, s>>>(
            inst, ntot, (const float4*)pos_a, (const float4*)pos_b, (const float4*)frc, grid);
    else
        k_spread<T, Dbl4, Dbl4><<<blocks, kSpreadWarps * 32, 0, s>>>(
            inst, ntot, (const Dbl4*)pos_a, (const Dbl4*)pos_b, (const Dbl4*)frc, grid);
}

template <class T>
void launch_gather(const PbInst* inst, int ninst, const int* tgt_offsets, int ncap, const void* pos_a,
                   const void* pos_b, const T* grid, T* u_k, cudaStream_t s)
{
    if (ncap <= 0) return;
    int blocks = (ncap + kSpreadWarps - 1) / kSpreadWarps;
    const int* ntot = tgt_offsets + ninst;
    if (sizeof(T) == 4)
        k_gather<T, float4><<<blocks, kSpreadWarps * 32, 0, s>>>(inst, ntot, (const float4*)pos_a,
                                                                   (const float4*)pos_b, grid, u_k);
    else
        k_gather<T, Dbl4><<<blocks, kSpreadWarps * 32, 0, s>>>(inst, ntot, (const Dbl4*)pos_a,
                                                                    (const Dbl4*)pos_b, grid, u_k);
}

template void launch_spread<float>(const PbInst*, int, const int*, int, const void*, const void*, const void*, float*,
                                   cudaStream_t);
template void launch_spread<double>(const PbInst*, int, const int*, int, const void*, const void*, const void*,
                                    double*, cudaStream_t);
template void launch_gather<float>(const PbInst*, int, const int*, int, const void*, const void*, const float*,
                                   float*, cudaStream_t);
template void launch_gather<double>(const PbInst*, int, const int*, int, const void*, const void*, const double*,
                                    double*, cudaStream_t);

// ---------------------------------------------------------------------------
// Shared-memory Stockham FFT (radix 2)
// ---------------------------------------------------------------------------
// Transforms `nl` lines of length N held in smem: element (l, i) at
// buf[l*ls + i*es].  Forward uses W_N^k = exp(-2 pi i k/N) from tw[k] (k < N/2);
// inverse conjugates.  Unnormalised.  Returns the buffer holding the result.
// Thread mapping: `lfast` puts the line index in the fastest thread dimension
// (use when es == 1 is false, i.e. lines interleaved).
template <class T2>
__device__ T2* stockham(T2* a, T2* b, int N, int nl, int ls, int es, const T2* __restrict__ tw, bool inverse,
                        bool lfast)
{
    const int half = N >> 1;
    const int total = nl * half;
    for (int Ns = 1; Ns < N; Ns <<= 1) {
        const int tstep = N / (2 * Ns);
        for (int wdx = threadIdx.x; wdx < total; wdx += blockDim.x) {
            int l, j;
            if (lfast) {
                l = wdx % nl;
                j = wdx / nl;
            } else {
                j = wdx % half;
                l = wdx / half;
            }
            T2 a0 = a[l * ls + j * es], a1 = a[l * ls + (j + half) * es];
            int k = j & (Ns - 1);
            T2 w = tw[k * tstep];
            if (inverse) w.y = -w.y;
            a1 = cmul(a1, w);
            int di = ((j - k) << 1) + k;
            T2 s, d;
            s.x = a0.x + a1.x;
            s.y = a0.y + a1.y;
            d.x = a0.x - a1.x;
            d.y = a0.y - a1.y;
            b[l * ls + di * es] = s;
            b[l * ls + (di + Ns) * es] = d;
        }
        __syncthreads();
        T2* t = a;
        a = b;
        b = t;
    }
    return a;
}

// Twiddle table layout for one grid bucket (M = {Mx, My, Mz}, Nh = Mz/2):
//   [W_Nh: Nh/2][W_My: My/2][W_Mx: Mx/2][R: Nh+1 with R_k = exp(-2 pi i k / Mz)]
struct TwOff {
    int zh, y, x, r, total;
};
__host__ __device__ inline TwOff tw_offsets(const int* M)
{
    TwOff o;
    int Nh = M[2] / 2;
    o.zh = 0;
    o.y = o.zh + (Nh / 2 > 0 ? Nh / 2 : 1);
    o.x = o.y + M[1] / 2;
    o.r = o.x + M[0] / 2;
    o.total = o.r + Nh + 1;
    return o;
}

size_t twiddle_bytes(const int* M, bool fp64)
{
    return (size_t)tw_offsets(M).total * (fp64 ? sizeof(double2) : sizeof(float2));
}

void fill_twiddles(const int* M, bool fp64, void* host_buf)
{
    TwOff o = tw_offsets(M);
    int Nh = M[2] / 2;
    auto put = [&](int at, double ang) {
        double c = cos(ang), s = sin(ang);
        if (fp64) {
            ((double2*)host_buf)[at] = make_double2(c, s);
        } else {
            ((float2*)host_buf)[at] = make_float2((float)c, (float)s);
        }
    };
    for (int k = 0; k < (Nh / 2 > 0 ? Nh / 2 : 1); k++) put(o.zh + k, -2 * kPiD * k / (Nh > 0 ? Nh : 1));
    for (int k = 0; k < M[1] / 2; k++) put(o.y + k, -2 * kPiD * k / M[1]);
    for (int k = 0; k < M[0] / 2; k++) put(o.x + k, -2 * kPiD * k / M[0]);
    for (int k = 0; k <= Nh; k++) put(o.r + k, -2 * kPiD * k / M[2]);
}

// z pass, forward: real lines of length Mz -> Nh+1 complex (packed half-length FFT).
template <class T>
__global__ void k_fft_z_fwd(const T* __restrict__ grid, typename Cx<T>::t* __restrict__ spec, long long nlines, int Mz,
                            int lpb, const typename Cx<T>::t* __restrict__ tw, TwOff o)
{
    typedef typename Cx<T>::t T2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2* A = (T2*)smem_raw;
    const int Nh = Mz / 2, Mzh = Nh + 1;
    T2* B = A + lpb * Nh;
    long long l0 = (long long)blockIdx.x * lpb;
    int nl = (int)min((long long)lpb, nlines - l0);
    for (int idx = threadIdx.x; idx < nl * Nh; idx += blockDim.x) {
        int l = idx / Nh, i = idx - l * Nh;
        const T2* src = (const T2*)(grid + (size_t)(l0 + l) * Mz);
        A[l * Nh + i] = src[i];
    }
    __syncthreads();
    T2* R = (Nh > 1) ? stockham<T2>(A, B, Nh, nl, Nh, 1, tw + o.zh, false, false) : A;
    const T2* rt = tw + o.r;
    for (int idx = threadIdx.x; idx < nl * Mzh; idx += blockDim.x) {
        int l = idx / Mzh, k = idx - l * Mzh;
        T2 zk = R[l * Nh + (k == Nh ? 0 : k)];
        T2 zm = R[l * Nh + (k == 0 ? 0 : Nh - k)];
        // E = (zk + conj(zm))/2, O = (zk - conj(zm))/(2i)
        T2 E, Od;
        E.x = (T)0.5 * (zk.x + zm.x);
        E.y = (T)0.5 * (zk.y - zm.y);
        Od.x = (T)0.5 * (zk.y + zm.y);
        Od.y = (T)-0.5 * (zk.x - zm.x);
        T2 wo = cmul(rt[k], Od);
        T2 X;
        X.x = E.x + wo.x;
        X.y = E.y + wo.y;
        spec[(size_t)(l0 + l) * Mzh + k] = X;
    }
}

// z pass, inverse: Nh+1 complex -> real line of length Mz.
template <class T>
__global__ void k_fft_z_inv(const typename Cx<T>::t* __restrict__ spec, T* __restrict__ grid, long long nlines, int Mz,
                            int lpb, const typename Cx<T>::t* __restrict__ tw, TwOff o)
{
    typedef typename Cx<T>::t T2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2* A = (T2*)smem_raw;
    const int Nh = Mz / 2, Mzh = Nh + 1;
    T2* B = A + lpb * Nh;
    const T2* rt = tw + o.r;
    long long l0 = (long long)blockIdx.x * lpb;
    int nl = (int)min((long long)lpb, nlines - l0);
    for (int idx = threadIdx.x; idx < nl * Nh; idx += blockDim.x) {
        int l = idx / Nh, k = idx - l * Nh;
        const T2* src = spec + (size_t)(l0 + l) * Mzh;
        T2 xk = src[k], xm = src[Nh - k];
        // Z_k = (xk + conj(xm)) + i W^{-k} (xk - conj(xm))
        T2 e, dlt;
        e.x = xk.x + xm.x;
        e.y = xk.y - xm.y;
        dlt.x = xk.x - xm.x;
        dlt.y = xk.y + xm.y;
        T2 wc = rt[k];
        wc.y = -wc.y;
        T2 od = cmul(wc, dlt);
        T2 Z;
        Z.x = e.x - od.y;
        Z.y = e.y + od.x;
        A[l * Nh + k] = Z;
    }
    __syncthreads();
    T2* R = (Nh > 1) ? stockham<T2>(A, B, Nh, nl, Nh, 1, tw + o.zh, true, false) : A;
    for (int idx = threadIdx.x; idx < nl * Nh; idx += blockDim.x) {
        int l = idx / Nh, i = idx - l * Nh;
        T2* dst = (T2*)(grid + (size_t)(l0 + l) * Mz);
        dst[i] = R[l * Nh + i];
    }
}

// y pass (forward or inverse) over volumes [nvol][Mx][My][Mzh]; tile of TW z' columns.
template <class T>
__global__ void k_fft_y(typename Cx<T>::t* __restrict__ spec, int nvol, int Mx, int My, int Mzh, int TW,
                        const typename Cx<T>::t* __restrict__ tw, int tw_off, bool inverse)
{
    typedef typename Cx<T>::t T2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2* A = (T2*)smem_raw;
    T2* B = A + TW * My;
    const int ntile = (Mzh + TW - 1) / TW;
    long long blk = blockIdx.x;
    int tile = (int)(blk % ntile);
    long long vx = blk / ntile;  // vol*Mx + x
    int z0 = tile * TW;
    int nl = min(TW, Mzh - z0);
    T2* base = spec + (size_t)vx * My * Mzh + z0;
    for (int idx = threadIdx.x; idx < My * TW; idx += blockDim.x) {
        int i = idx / TW, l = idx - i * TW;
        if (l < nl) A[i * TW + l] = base[(size_t)i * Mzh + l];
    }
    __syncthreads();
    T2* R = stockham<T2>(A, B, My, TW, 1, TW, tw + tw_off, inverse, true);
    for (int idx = threadIdx.x; idx < My * TW; idx += blockDim.x) {
        int i = idx / TW, l = idx - i * TW;
        if (l < nl) base[(size_t)i * Mzh + l] = R[i * TW + l];
    }
}

// x pass fused: forward FFT along x of the three components, Green tensor
// multiply, inverse FFT along x.  One block per (instance, y, z'-tile).
struct GreenConst {
    double twopi_L[3];
    double a2, a1_over_a2, gexp, kfac;  // kfac * (1 + a1 k^2/a^2) exp(-k^2 gexp) / (k^2 (k^2 + a^2))
};

template <class T>
__global__ void k_fft_x_green(typename Cx<T>::t* __restrict__ spec, const PbInst* __restrict__ inst,
                              const int* __restrict__ bucket_inst, long long base_off, int Mx, int My, int Mzh, int Mz,
                              int TW, const typename Cx<T>::t* __restrict__ tw, int tw_off)
{
    typedef typename Cx<T>::t T2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2* A = (T2*)smem_raw;
    T2* B = A + 3 * TW * Mx;
    const int ntile = (Mzh + TW - 1) / TW;
    long long blk = blockIdx.x;
    int tile = (int)(blk % ntile);
    long long r = blk / ntile;
    int y = (int)(r % My);
    int qi = (int)(r / My);
    const PbInst& I = inst[bucket_inst[qi]];
    int z0 = tile * TW;
    int nl = min(TW, Mzh - z0);
    const size_t vol = (size_t)Mx * My * Mzh;
    T2* base = spec + (I.spec_off - base_off) + (size_t)y * Mzh + z0;
    // smem layout: line (c, l) at (c*TW + l), element i stride 3*TW
    const int NL = 3 * TW;
    for (int idx = threadIdx.x; idx < 3 * Mx * TW; idx += blockDim.x) {
        int l = idx % TW, rest = idx / TW, i = rest % Mx, c = rest / Mx;
        if (l < nl) A[i * NL + c * TW + l] = base[c * vol + (size_t)i * My * Mzh + l];
    }
    __syncthreads();
    T2* R = stockham<T2>(A, B, Mx, NL, 1, NL, tw + tw_off, false, true);
    T2* S = (R == A) ? B : A;
    // Green multiply in place in R
    const double tpx = 2 * kPiD / I.L[0], tpy = 2 * kPiD / I.L[1], tpz = 2 * kPiD / I.L[2];
    const double a2 = I.alpha * I.alpha;
    const T a1oa2 = (T)(-expm1(-a2 * I.d * I.d / 4) / a2);
    const T gexp = (T)(I.d * I.d / 4 - I.eta / 2);
    const T kfac = (T)I.kfac;
    const int My_ = My;
    int ny = (y < My_ / 2) ? y : y - My_;
    bool ynyq = (2 * y == My_);
    for (int idx = threadIdx.x; idx < Mx * TW; idx += blockDim.x) {
        int l = idx % TW, i = idx / TW;
        if (l >= nl) continue;
        int kz = z0 + l;
        int nx = (i < Mx / 2) ? i : i - Mx;
        bool zero = (2 * i == Mx) || ynyq || (2 * kz == Mz) || (nx == 0 && ny == 0 && kz == 0);
        T2* v0 = &R[i * NL + 0 * TW + l];
        T2* v1 = &R[i * NL + 1 * TW + l];
        T2* v2 = &R[i * NL + 2 * TW + l];
        if (zero) {
            *v0 = T2{0, 0};
            *v1 = T2{0, 0};
            *v2 = T2{0, 0};
            continue;
        }
        T kx = (T)(tpx * nx), ky = (T)(tpy * ny), kzv = (T)(tpz * kz);
        T kn = kx * kx + ky * ky + kzv * kzv;
        T s = kfac * ((T)1 + a1oa2 * kn) * exp(-kn * gexp) / (kn * (kn + (T)a2));
        T2 A0 = *v0, A1 = *v1, A2 = *v2;
        T dr = kx * A0.x + ky * A1.x + kzv * A2.x;
        T di = kx * A0.y + ky * A1.y + kzv * A2.y;
        *v0 = T2{s * (kn * A0.x - kx * dr), s * (kn * A0.y - kx * di)};
        *v1 = T2{s * (kn * A1.x - ky * dr), s * (kn * A1.y - ky * di)};
        *v2 = T2{s * (kn * A2.x - kzv * dr), s * (kn * A2.y - kzv * di)};
    }
    __syncthreads();
    T2* R2 = stockham<T2>(R, S, Mx, NL, 1, NL, tw + tw_off, true, true);
    for (int idx = threadIdx.x; idx < 3 * Mx * TW; idx += blockDim.x) {
        int l = idx % TW, rest = idx / TW, i = rest % Mx, c = rest / Mx;
        if (l < nl) base[c * vol + (size_t)i * My * Mzh + l] = R2[i * NL + c * TW + l];
    }
}

static int pick_tw(int N, int mult, size_t csize, int maxbytes)
{
    int tw = 16;
    while (tw > 1 && (size_t)2 * mult * tw * N * csize > (size_t)maxbytes) tw >>= 1;
    return tw;
}

template <class T>
void launch_kspace_fft(const PbInst* inst_dev, const int* bucket_inst, int nb, long long base_off, const int* M,
                       T* grid, void* spec_v, const void* tw_v, cudaStream_t s)
{
    typedef typename Cx<T>::t T2;
    T2* spec = (T2*)spec_v;
    const T2* tw = (const T2*)tw_v;
    const int Mx = M[0], My = M[1], Mz = M[2], Nh = Mz / 2, Mzh = Nh + 1;
    const int nvol = 3 * nb;
    TwOff o = tw_offsets(M);
    const size_t cs = sizeof(T2);
    const int smax = 64 * 1024;
    // z forward
    long long nlines = (long long)nvol * Mx * My;
    int lpb = (int)(2048 / (Nh > 0 ? Nh : 1));
    if (lpb < 1) lpb = 1;
    size_t sm = (size_t)2 * lpb * Nh * cs;
    cudaFuncSetAttribute(k_fft_z_fwd<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_fft_z_fwd<T><<<(unsigned)((nlines + lpb - 1) / lpb), 256, sm, s>>>(grid, spec, nlines, Mz, lpb, tw, o);
    // y forward
    int twy = pick_tw(My, 1, cs, smax);
    size_t smy = (size_t)2 * twy * My * cs;
    cudaFuncSetAttribute(k_fft_y<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smy);
    long long nby = (long long)nvol * Mx * ((Mzh + twy - 1) / twy);
    k_fft_y<T><<<(unsigned)nby, 256, smy, s>>>(spec, nvol, Mx, My, Mzh, twy, tw, o.y, false);
    // x forward + Green + x inverse
    int twx = pick_tw(Mx, 3, cs, smax);
    size_t smx = (size_t)2 * 3 * twx * Mx * cs;
    cudaFuncSetAttribute(k_fft_x_green<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smx);
    long long nbx = (long long)nb * My * ((Mzh + twx - 1) / twx);
    k_fft_x_green<T><<<(unsigned)nbx, 256, smx, s>>>(spec, inst_dev, bucket_inst, base_off, Mx, My, Mzh, Mz, twx, tw,
                                                       o.x);
    // y inverse
    k_fft_y<T><<<(unsigned)nby, 256, smy, s>>>(spec, nvol, Mx, My, Mzh, twy, tw, o.y, true);
    // z inverse
    cudaFuncSetAttribute(k_fft_z_inv<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_fft_z_inv<T><<<(unsigned)((nlines + lpb - 1) / lpb), 256, sm, s>>>(spec, grid, nlines, Mz, lpb, tw, o);
}

template void launch_kspace_fft<float>(const PbInst*, const int*, int, long long, const int*, float*, void*,
                                       const void*, cudaStream_t);
template void launch_kspace_fft<double>(const PbInst*, const int*, int, long long, const int*, double*, void*,
                                        const void*, cudaStream_t);

// ---------------------------------------------------------------------------
// Final FP64 combine and force sums
// ---------------------------------------------------------------------------
__global__ void k_combine_mixed(const PbInst* __restrict__ inst, int ninst, const int* __restrict__ tgt_offsets,
                                const int* __restrict__ tperm, const float* __restrict__ u_s,
                                const float* __restrict__ u_c, const double* __restrict__ u_near,
                                const float* __restrict__ u_k, int use_real, int use_k, const double* __restrict__ fsum,
                                const PbTables* __restrict__ tab, const double* __restrict__ frc,
                                const int* __restrict__ src_offsets, double* __restrict__ U)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tgt_offsets[ninst]) return;
    int p = tperm[t];
    int q = find_instance(tgt_offsets, ninst, p);
    const PbInst& I = inst[q];
    double tau = I.L[0] * I.L[1] * I.L[2];
    // self pair (targets are the sources): (R_eps(0) - R_d(0)) f_i in FP64
    const bool self = use_real && I.same && (I.flags & 1);
    const size_t ps = (size_t)(p - tgt_offsets[q] + src_offsets[q]);
    for (int c = 0; c < 3; c++) {
        double v = 0;
        size_t o = 3 * (size_t)t + c;
        if (self) v += tab[q].self1 * frc[3 * ps + c];
        if (use_real && (I.flags & 1)) v += ((double)u_s[o] - (double)u_c[o]) + u_near[o];
        if (use_k && (I.flags & 2)) v += (double)u_k[o];
        if (I.flags & 4) v += fsum[3 * q + c] / (I.alpha * I.alpha * tau);
        U[3 * (size_t)p + c] = v;
    }
}

__global__ void k_combine_fp64(const PbInst* __restrict__ inst, int ninst, const int* __restrict__ tgt_offsets,
                               const int* __restrict__ tperm, const double* __restrict__ u_real,
                               const double* __restrict__ u_k, int use_real, int use_k,
                               const double* __restrict__ fsum, const PbTables* __restrict__ tab,
                               const double* __restrict__ frc, const int* __restrict__ src_offsets,
                               double* __restrict__ U)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tgt_offsets[ninst]) return;
    int p = tperm[t];
    int q = find_instance(tgt_offsets, ninst, p);
    const PbInst& I = inst[q];
    double tau = I.L[0] * I.L[1] * I.L[2];
    const bool self = use_real && I.same && (I.flags & 1);
    const size_t ps = (size_t)(p - tgt_offsets[q] + src_offsets[q]);
    for (int c = 0; c < 3; c++) {
        double v = 0;
        size_t o = 3 * (size_t)t + c;
        if (self) v += tab[q].self1 * frc[3 * ps + c];
        if (use_real && (I.flags & 1)) v += u_real[o];
        if (use_k && (I.flags & 2)) v += u_k[o];
        if (I.flags & 4) v += fsum[3 * q + c] / (I.alpha * I.alpha * tau);
        U[3 * (size_t)p + c] = v;
    }
}

void launch_combine_mixed(const PbInst* inst, int ninst, const int* tgt_offsets, int ncap, const int* tperm,
                          const float* u_s, const float* u_c, const double* u_near, const float* u_k, int use_real,
                          int use_k, const double* fsum, const PbTables* tab, const double* frc,
                          const int* src_offsets, double* U, cudaStream_t s)
{
    if (ncap <= 0) return;
    k_combine_mixed<<<(ncap + 255) / 256, 256, 0, s>>>(inst, ninst, tgt_offsets, tperm, u_s, u_c, u_near, u_k,
                                                        use_real, use_k, fsum, tab, frc, src_offsets, U);
}

void launch_combine_fp64(const PbInst* inst, int ninst, const int* tgt_offsets, int ncap, const int* tperm,
                         const double* u_real, const double* u_k, int use_real, int use_k, const double* fsum,
                         const PbTables* tab, const double* frc, const int* src_offsets, double* U, cudaStream_t s)
{
    if (ncap <= 0) return;
    k_combine_fp64<<<(ncap + 255) / 256, 256, 0, s>>>(inst, ninst, tgt_offsets, tperm, u_real, u_k, use_real,
                                                       use_k, fsum, tab, frc, src_offsets, U);
}

__global__ void k_force_sums(const double* __restrict__ frc, const int* __restrict__ offsets, int ninst,
                             double* __restrict__ out)
{
    int q = blockIdx.x;
    if (q >= ninst) return;
    int b = offsets[q], e = offsets[q + 1];
    double s[3] = {0, 0, 0};
    for (int p = b + threadIdx.x; p < e; p += blockDim.x)
        for (int c = 0; c < 3; c++) s[c] += frc[3 * (size_t)p + c];
    __shared__ double red[3][256];
    for (int c = 0; c < 3; c++) red[c][threadIdx.x] = s[c];
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st)
            for (int c = 0; c < 3; c++) red[c][threadIdx.x] += red[c][threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int c = 0; c < 3; c++) out[3 * q + c] = red[c][0];
}

void launch_force_sums(const double* frc, const int* offsets, int ninst, double* out, cudaStream_t s)
{
    if (ninst <= 0) return;
    k_force_sums<<<ninst, 256, 0, s>>>(frc, offsets, ninst, out);
}

}  // namespace pb

// ---------------------------------------------------------------------------
// Tiled spreading and gathering
// ---------------------------------------------------------------------------
// A tile is a block of ublk^3 real-space cells; its particles are contiguous
// z-runs of the cell-sorted arrays.  The union of their Gaussian windows is a
// small box of the grid held in shared memory: spreading accumulates every
// particle into it with plain read-modify-writes (the whole block works on one
// particle at a time, each thread on distinct points) and adds the box to the
// global grid once; gathering loads the box once and every warp interpolates
// its targets from shared memory.
namespace pb {

constexpr int kTileThreads = 512;

template <class T>
struct TileCap {
    static constexpr int points = sizeof(T) == 4 ? 10648 : 5832;  // 22^3 / 18^3 points, three components
};

struct TileGeom {
    int q, c0[3], c1[3];  // instance, cell range [c0, c1) per axis
    int lo[3], R[3];      // grid box origin (unwrapped) and size
};

__device__ __forceinline__ void tile_geom(const PbInst* __restrict__ inst, const int* __restrict__ unit_off, int ninst,
                                          int u, TileGeom& G)
{
    int q = find_instance(unit_off, ninst, u);
    const PbInst& I = inst[q];
    int local = u - unit_off[q];
    int uz = local % I.nu[2];
    int r = local / I.nu[2];
    int uy = r % I.nu[1], ux = r / I.nu[1];
    int uu[3] = {ux, uy, uz};
    G.q = q;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        G.c0[a] = uu[a] * I.ublk;
        G.c1[a] = min(G.c0[a] + I.ublk, I.nc[a]);
        double s = I.h[a] / I.gh[a];
        int f0 = (int)floor(G.c0[a] * s), f1 = (int)floor(G.c1[a] * s);
        G.lo[a] = f0 - I.Pa[a] / 2;  // one point of margin below the lowest window start
        G.R[a] = (f1 + I.Pa[a] / 2 + 1) - G.lo[a] + 1;
    }
}

template <class T, class PV, class FV>
__global__ void __launch_bounds__(kTileThreads)
    k_spread_tiles(const PbInst* __restrict__ inst, int ninst, const int* __restrict__ unit_off,
                   const int* __restrict__ cstart, const PV* __restrict__ pa, const PV* __restrict__ pb,
                   const FV* __restrict__ frc, T* __restrict__ grid)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* reg = (T*)smem_raw;
    __shared__ T wts[3][kMaxP];
    __shared__ int wst[3];
    __shared__ T fsh[3];
    __shared__ int inbox;
    const int total = unit_off[ninst];
    for (int u = blockIdx.x; u < total; u += gridDim.x) {
        TileGeom G;
        tile_geom(inst, unit_off, ninst, u, G);
        const PbInst& I = inst[G.q];
        const int R = G.R[0] * G.R[1] * G.R[2];
        // any particles in the tile?
        int cnt = 0;
        for (int cx = G.c0[0]; cx < G.c1[0]; cx++)
            for (int cy = G.c0[1]; cy < G.c1[1]; cy++) {
                int row = I.cell_off + (cx * I.nc[1] + cy) * I.nc[2];
                cnt += cstart[row + G.c1[2]] - cstart[row + G.c0[2]];
            }
        if (cnt == 0) continue;
        const bool boxed = R <= TileCap<T>::points;
        if (boxed)
            for (int i = threadIdx.x; i < 3 * R; i += blockDim.x) reg[i] = (T)0;
        __syncthreads();
        const size_t comp = (size_t)I.M[0] * I.M[1] * I.M[2];
        T* g0 = grid + I.grid_off;
        const int Py = I.Pa[1], Pz = I.Pa[2], P2 = Py * Pz, P3 = I.Pa[0] * P2;
        for (int cx = G.c0[0]; cx < G.c1[0]; cx++)
            for (int cy = G.c0[1]; cy < G.c1[1]; cy++) {
                int row = I.cell_off + (cx * I.nc[1] + cy) * I.nc[2];
                int b = cstart[row + G.c0[2]], e = cstart[row + G.c1[2]];
                for (int s = b; s < e; s++) {
                    if (threadIdx.x < 3 * 32) {
                        int a = threadIdx.x >> 5, p = threadIdx.x & 31;
                        double x[3];
                        int qq;
                        load_pos(pa, pb, s, x, qq);
                        if (p < I.Pa[a]) {
                            double h = I.gh[a];
                            int gs = (int)floor(x[a] / h) - I.Pa[a] / 2 + 1;
                            T dx = (T)(x[a] - (double)(gs + p) * h);
                            wts[a][p] = exp(-dx * dx / (T)I.eta);
                            if (p == 0) wst[a] = gs - G.lo[a];
                        }
                        if (threadIdx.x == 0) {
                            double fv[3];
                            load_frc(frc, s, fv);
                            fsh[0] = (T)fv[0];
                            fsh[1] = (T)fv[1];
                            fsh[2] = (T)fv[2];
                        }
                    }
                    __syncthreads();
                    if (threadIdx.x == 0)
                        inbox = boxed && wst[0] >= 0 && wst[1] >= 0 && wst[2] >= 0 && wst[0] + I.Pa[0] <= G.R[0] &&
                                wst[1] + Py <= G.R[1] && wst[2] + Pz <= G.R[2];
                    __syncthreads();
                    const T f0 = fsh[0], f1 = fsh[1], f2 = fsh[2];
                    if (inbox) {
                        for (int id = threadIdx.x; id < P3; id += blockDim.x) {
                            int px = id / P2, rr = id - px * P2, py = rr / Pz, pz = rr - py * Pz;
                            T wv = wts[0][px] * wts[1][py] * wts[2][pz];
                            int ri = ((wst[0] + px) * G.R[1] + wst[1] + py) * G.R[2] + wst[2] + pz;
                            reg[ri] += f0 * wv;
                            reg[R + ri] += f1 * wv;
                            reg[2 * R + ri] += f2 * wv;
                        }
                    } else {  // window outside the box (or box too large): straight to the grid
                        for (int id = threadIdx.x; id < P3; id += blockDim.x) {
                            int px = id / P2, rr = id - px * P2, py = rr / Pz, pz = rr - py * Pz;
                            T wv = wts[0][px] * wts[1][py] * wts[2][pz];
                            int gx = (G.lo[0] + wst[0] + px) % I.M[0], gy = (G.lo[1] + wst[1] + py) % I.M[1],
                                gz = (G.lo[2] + wst[2] + pz) % I.M[2];
                            gx += gx < 0 ? I.M[0] : 0;
                            gy += gy < 0 ? I.M[1] : 0;
                            gz += gz < 0 ? I.M[2] : 0;
                            size_t o = ((size_t)gx * I.M[1] + gy) * I.M[2] + gz;
                            atomicAdd(g0 + o, f0 * wv);
                            atomicAdd(g0 + comp + o, f1 * wv);
                            atomicAdd(g0 + 2 * comp + o, f2 * wv);
                        }
                    }
                    __syncthreads();
                }
            }
        if (boxed) {
            for (int i = threadIdx.x; i < R; i += blockDim.x) {
                int iz = i % G.R[2], r2 = i / G.R[2], iy = r2 % G.R[1], ix = r2 / G.R[1];
                int gx = (G.lo[0] + ix) % I.M[0], gy = (G.lo[1] + iy) % I.M[1], gz = (G.lo[2] + iz) % I.M[2];
                gx += gx < 0 ? I.M[0] : 0;
                gy += gy < 0 ? I.M[1] : 0;
                gz += gz < 0 ? I.M[2] : 0;
                size_t o = ((size_t)gx * I.M[1] + gy) * I.M[2] + gz;
                T v0 = reg[i], v1 = reg[R + i], v2 = reg[2 * R + i];
                if (v0 != (T)0) atomicAdd(g0 + o, v0);
                if (v1 != (T)0) atomicAdd(g0 + comp + o, v1);
                if (v2 != (T)0) atomicAdd(g0 + 2 * comp + o, v2);
            }
        }
        __syncthreads();
    }
}

template <class T, class PV>
__global__ void __launch_bounds__(kTileThreads)
    k_gather_tiles(const PbInst* __restrict__ inst, int ninst, const int* __restrict__ unit_off,
                   const int* __restrict__ cstart, const PV* __restrict__ pa, const PV* __restrict__ pb,
                   const T* __restrict__ grid, T* __restrict__ u_k)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* reg = (T*)smem_raw;
    constexpr int NW = kTileThreads / 32;
    __shared__ T wts[NW][3][kMaxP];
    __shared__ int wst[NW][3];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int total = unit_off[ninst];
    for (int u = blockIdx.x; u < total; u += gridDim.x) {
        TileGeom G;
        tile_geom(inst, unit_off, ninst, u, G);
        const PbInst& I = inst[G.q];
        const int R = G.R[0] * G.R[1] * G.R[2];
        int cnt = 0;
        for (int cx = G.c0[0]; cx < G.c1[0]; cx++)
            for (int cy = G.c0[1]; cy < G.c1[1]; cy++) {
                int row = I.cell_off + (cx * I.nc[1] + cy) * I.nc[2];
                cnt += cstart[row + G.c1[2]] - cstart[row + G.c0[2]];
            }
        if (cnt == 0) continue;
        const bool boxed = R <= TileCap<T>::points;
        const size_t comp = (size_t)I.M[0] * I.M[1] * I.M[2];
        const T* g0 = grid + I.grid_off;
        if (boxed)
            for (int i = threadIdx.x; i < R; i += blockDim.x) {
                int iz = i % G.R[2], r2 = i / G.R[2], iy = r2 % G.R[1], ix = r2 / G.R[1];
                int gx = (G.lo[0] + ix) % I.M[0], gy = (G.lo[1] + iy) % I.M[1], gz = (G.lo[2] + iz) % I.M[2];
                gx += gx < 0 ? I.M[0] : 0;
                gy += gy < 0 ? I.M[1] : 0;
                gz += gz < 0 ? I.M[2] : 0;
                size_t o = ((size_t)gx * I.M[1] + gy) * I.M[2] + gz;
                reg[i] = g0[o];
                reg[R + i] = g0[comp + o];
                reg[2 * R + i] = g0[2 * comp + o];
            }
        __syncthreads();
        const int Py = I.Pa[1], Pz = I.Pa[2], P2 = Py * Pz, P3 = I.Pa[0] * P2;
        // the tile's targets, one warp each
        int k = 0;
        for (int cx = G.c0[0]; cx < G.c1[0]; cx++)
            for (int cy = G.c0[1]; cy < G.c1[1]; cy++) {
                int row = I.cell_off + (cx * I.nc[1] + cy) * I.nc[2];
                int b = cstart[row + G.c0[2]], e = cstart[row + G.c1[2]];
                for (int s = b; s < e; s++, k++) {
                    if ((k % NW) != w) continue;
                    double x[3];
                    int qq;
                    load_pos(pa, pb, s, x, qq);
#pragma unroll
                    for (int a = 0; a < 3; a++) {
                        if (lane < I.Pa[a]) {
                            double h = I.gh[a];
                            int gs = (int)floor(x[a] / h) - I.Pa[a] / 2 + 1;
                            T dx = (T)(x[a] - (double)(gs + lane) * h);
                            wts[w][a][lane] = exp(-dx * dx / (T)I.eta);
                            if (lane == 0) wst[w][a] = gs - G.lo[a];
                        }
                    }
                    __syncwarp();
                    const bool inbox = boxed && wst[w][0] >= 0 && wst[w][1] >= 0 && wst[w][2] >= 0 &&
                                       wst[w][0] + I.Pa[0] <= G.R[0] && wst[w][1] + Py <= G.R[1] &&
                                       wst[w][2] + Pz <= G.R[2];
                    T s0 = 0, s1 = 0, s2 = 0, e0 = 0, e1 = 0, e2 = 0;
                    for (int id = lane; id < P3; id += 32) {
                        int px = id / P2, rr = id - px * P2, py = rr / Pz, pz = rr - py * Pz;
                        T wv = wts[w][0][px] * wts[w][1][py] * wts[w][2][pz];
                        T v0, v1, v2;
                        if (inbox) {
                            int ri = ((wst[w][0] + px) * G.R[1] + wst[w][1] + py) * G.R[2] + wst[w][2] + pz;
                            v0 = reg[ri];
                            v1 = reg[R + ri];
                            v2 = reg[2 * R + ri];
                        } else {
                            int gx = (G.lo[0] + wst[w][0] + px) % I.M[0], gy = (G.lo[1] + wst[w][1] + py) % I.M[1],
                                gz = (G.lo[2] + wst[w][2] + pz) % I.M[2];
                            gx += gx < 0 ? I.M[0] : 0;
                            gy += gy < 0 ? I.M[1] : 0;
                            gz += gz < 0 ? I.M[2] : 0;
                            size_t o = ((size_t)gx * I.M[1] + gy) * I.M[2] + gz;
                            v0 = g0[o];
                            v1 = g0[comp + o];
                            v2 = g0[2 * comp + o];
                        }
                        T y = wv * v0 - e0, t = s0 + y;
                        e0 = (t - s0) - y;
                        s0 = t;
                        y = wv * v1 - e1;
                        t = s1 + y;
                        e1 = (t - s1) - y;
                        s1 = t;
                        y = wv * v2 - e2;
                        t = s2 + y;
                        e2 = (t - s2) - y;
                        s2 = t;
                    }
                    s0 -= e0;
                    s1 -= e1;
                    s2 -= e2;
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) {
                        s0 += __shfl_xor_sync(kFull, s0, o);
                        s1 += __shfl_xor_sync(kFull, s1, o);
                        s2 += __shfl_xor_sync(kFull, s2, o);
                    }
                    if (lane == 0) {
                        u_k[3 * (size_t)s] = s0;
                        u_k[3 * (size_t)s + 1] = s1;
                        u_k[3 * (size_t)s + 2] = s2;
                    }
                    __syncwarp();
                }
            }
        __syncthreads();
    }
}

int tile_edge_points(bool fp64) { return fp64 ? 18 : 22; }

template <class T>
void launch_spread_tiles(const PbInst* inst, int ninst, const int* unit_off, int ucap, const int* cstart,
                         const void* pos_a, const void* pos_b, const void* frc, T* grid, int nsm, cudaStream_t s)
{
    if (ucap <= 0) return;
    size_t smem = (size_t)3 * TileCap<T>::points * sizeof(T);
    int blocks = std::min(ucap, nsm);
    if (sizeof(T) == 4) {
        cudaFuncSetAttribute(k_spread_tiles<T, float4, float4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_spread_tiles<T, float4, float4><<<blocks, kTileThreads, smem, s>>>(
            inst, ninst, unit_off, cstart, (const float4*)pos_a, (const float4*)pos_b, (const float4*)frc, grid);
    } else {
        cudaFuncSetAttribute(k_spread_tiles<T, Dbl4, Dbl4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_spread_tiles<T, Dbl4, Dbl4><<<blocks, kTileThreads, smem, s>>>(
            inst, ninst, unit_off, cstart, (const Dbl4*)pos_a, (const Dbl4*)pos_b, (const Dbl4*)frc, grid);
    }
}

template <class T>
void launch_gather_tiles(const PbInst* inst, int ninst, const int* unit_off, int ucap, const int* cstart,
                         const void* pos_a, const void* pos_b, const T* grid, T* u_k, int nsm, cudaStream_t s)
{
    if (ucap <= 0) return;
    size_t smem = (size_t)3 * TileCap<T>::points * sizeof(T);
    int blocks = std::min(ucap, nsm);
    if (sizeof(T) == 4) {
        cudaFuncSetAttribute(k_gather_tiles<T, float4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_gather_tiles<T, float4><<<blocks, kTileThreads, smem, s>>>(inst, ninst, unit_off, cstart,
                                                                      (const float4*)pos_a, (const float4*)pos_b, grid,
                                                                      u_k);
    } else {
        cudaFuncSetAttribute(k_gather_tiles<T, Dbl4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_gather_tiles<T, Dbl4><<<blocks, kTileThreads, smem, s>>>(inst, ninst, unit_off, cstart, (const Dbl4*)pos_a,
                                                                     (const Dbl4*)pos_b, grid, u_k);
    }
}

template void launch_spread_tiles<float>(const PbInst*, int, const int*, int, const int*, const void*, const void*,
                                         const void*, float*, int, cudaStream_t);
template void launch_spread_tiles<double>(const PbInst*, int, const int*, int, const int*, const void*, const void*,
                                          const void*, double*, int, cudaStream_t);
template void launch_gather_tiles<float>(const PbInst*, int, const int*, int, const int*, const void*, const void*,
                                         const float*, float*, int, cudaStream_t);
template void launch_gather_tiles<double>(const PbInst*, int, const int*, int, const int*, const void*, const void*,
                                          const double*, double*, int, cudaStream_t);

}  // namespace pb

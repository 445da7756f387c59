/*
 * Launcher of the reference's own CUDA kernels (TEST INFRASTRUCTURE ONLY).
 *
 * Loads the device image oracle/_ref/ref_kernels.cubin (or its PTX twin),
 * built by oracle/build_ref.sh from the reference's cuda/periodicBrinkman.h,
 * with the CUDA driver API into the current (primary) context, and launches
 * kernelFourier and kernelReal with the launch configuration of the
 * reference's periodicBrinkman() (cuda/periodicBrinkman.h:432-513), restated
 * here step by step: per-axis shell counts from the sorted box
 * (457-487), grid (chooseSize(m), chooseSize(n)), power-of-two block of at
 * most maxBlockSize threads covering the shell box, blockSize*9 doubles of
 * dynamic shared memory, kernelFourier first, then kernelReal.  Device
 * pointers in; dA (3m x 3n column-major) is accumulated into, as the
 * reference does.  Used to check the dense drop-in against the reference's
 * own compiled kernels on the GPU, and to time them.
 */
#include <cuda.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

// The kernel parameter layout of the stand-in matrix.h's MatrixOnDevice.
struct MatrixOnDevice {
    double* p;
    int r, c;
};

CUmodule g_mod = nullptr;
CUfunction g_real = nullptr, g_four = nullptr;
char g_err[512];

int fail(const char* what, CUresult r)
{
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    std::snprintf(g_err, sizeof(g_err), "%s: %s", what, s ? s : "?");
    return (int)r ? (int)r : -1;
}

// The stand-in matrix.h's chooseSize: the power of two >= n, capped at 2^maxBit.
unsigned choose_size(unsigned n, unsigned max_bit = 16)
{
    unsigned s = 1;
    while (s < n && s < (1u << max_bit)) s <<= 1;
    return s;
}

}  // namespace

extern "C" {

const char* refk_error(void) { return g_err; }

// Loads the image at `path` (cubin or NUL-terminated PTX) into the current
// context, or device 0's primary context when none is current.
int refk_load(const char* path)
{
    CUresult r = cuInit(0);
    if (r != CUDA_SUCCESS) return fail("cuInit", r);
    CUcontext ctx = nullptr;
    cuCtxGetCurrent(&ctx);
    if (!ctx) {
        CUdevice dev;
        if ((r = cuDeviceGet(&dev, 0)) != CUDA_SUCCESS) return fail("cuDeviceGet", r);
        if ((r = cuDevicePrimaryCtxRetain(&ctx, dev)) != CUDA_SUCCESS) return fail("cuDevicePrimaryCtxRetain", r);
        if ((r = cuCtxSetCurrent(ctx)) != CUDA_SUCCESS) return fail("cuCtxSetCurrent", r);
    }
    FILE* fp = std::fopen(path, "rb");
    if (!fp) {
        std::snprintf(g_err, sizeof(g_err), "cannot open %s", path);
        return -1;
    }
    std::vector<char> buf;
    char tmp[65536];
    size_t k;
    while ((k = std::fread(tmp, 1, sizeof(tmp), fp)) > 0) buf.insert(buf.end(), tmp, tmp + k);
    std::fclose(fp);
    buf.push_back('\0');
    if (g_mod) cuModuleUnload(g_mod);
    g_mod = nullptr;
    if ((r = cuModuleLoadData(&g_mod, buf.data())) != CUDA_SUCCESS) return fail("cuModuleLoadData", r);
    // kernelReal(MatrixOnDevice x3, double x3, int x3, double x3, uint) and
    // kernelFourier(..., int): their C++ (Itanium ABI) symbol names
    if ((r = cuModuleGetFunction(&g_real, g_mod, "_Z10kernelReal14MatrixOnDeviceS_S_dddiiidddj")) != CUDA_SUCCESS)
        return fail("kernelReal", r);
    if ((r = cuModuleGetFunction(&g_four, g_mod, "_Z13kernelFourier14MatrixOnDeviceS_S_dddiiidddi")) != CUDA_SUCCESS)
        return fail("kernelFourier", r);
    return 0;
}

// periodicBrinkman(dA, dx, dx0, a, d, e, M, N, L, maxBlockSize) on the
// reference's kernels; waits for them.  Returns 0 or a CUresult.
int refk_periodic_brinkman(double* dA, const double* dx, int m, const double* dx0, int n, double a, double d,
                           double e, int M, int N, const double* L, int maxBlockSize)
{
    if (!g_real || !g_four) {
        std::snprintf(g_err, sizeof(g_err), "reference kernels not loaded");
        return -1;
    }
    if (m <= 0 || n <= 0 || maxBlockSize <= 0 || maxBlockSize > 512) {
        std::snprintf(g_err, sizeof(g_err), "bad sizes (m, n > 0, 0 < maxBlockSize <= 512)");
        return -1;
    }
    unsigned max_bit = 0;
    while ((1u << max_bit) < (unsigned)maxBlockSize) max_bit++;
    if ((1u << max_bit) != (unsigned)maxBlockSize) max_bit--;
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
    // gridDim.y is limited to 65535: the kernels stride over columns, so a
    // smaller grid covers the same pairs
    unsigned gx = choose_size((unsigned)m), gy = choose_size((unsigned)n);
    if (gy > 32768) gy = 32768;
    MatrixOnDevice A{dA, 3 * m, 3 * n}, X{const_cast<double*>(dx), 3, m}, X0{const_cast<double*>(dx0), 3, n};
    double Lx = L[0], Ly = L[1], Lz = L[2];
    CUresult r;
    if (N > 0) {
        unsigned bs = choose_size((unsigned)((2 * Nx[0] + 1) * (2 * Nx[1] + 1) * (2 * Nx[2] + 1)), max_bit);
        int bit = 0;
        while ((1u << bit) < bs) bit++;
        void* args[] = {&A, &X, &X0, &a, &d, &e, &Nx[0], &Nx[1], &Nx[2], &Lx, &Ly, &Lz, &bit};
        r = cuLaunchKernel(g_four, gx, gy, 1, bs, 1, 1, bs * 9 * sizeof(double), nullptr, args, nullptr);
        if (r != CUDA_SUCCESS) return fail("kernelFourier launch", r);
    }
    if (M >= 0) {
        unsigned bs = choose_size((unsigned)((2 * Mx[0] + 1) * (2 * Mx[1] + 1) * (2 * Mx[2] + 1)), max_bit);
        unsigned bit = 0;
        while ((1u << bit) < bs) bit++;
        void* args[] = {&A, &X, &X0, &a, &d, &e, &Mx[0], &Mx[1], &Mx[2], &Lx, &Ly, &Lz, &bit};
        r = cuLaunchKernel(g_real, gx, gy, 1, bs, 1, 1, bs * 9 * sizeof(double), nullptr, args, nullptr);
        if (r != CUDA_SUCCESS) return fail("kernelReal launch", r);
    }
    if ((r = cuCtxSynchronize()) != CUDA_SUCCESS) return fail("cuCtxSynchronize", r);
    return 0;
}

}  // extern "C"

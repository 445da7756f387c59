// A caller written against the reference's interface (TEST PROGRAM): the
// reference's matrix types (here the stand-in of its matrix library,
// oracle/ref_shim/include/matrix.h), its readData calls with its driver's
// defaults (cuda/periodicBrinkman.cu:78-92), and periodicBrinkman /
// fftBrinkman with their reference signatures, compiled unchanged against
// include/pbrinkman.hpp.  Usage: reference_caller param.txt [gpu]
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "matrix.h"
#include "pbrinkman.hpp"

int main(int argc, char** argv)
{
    if (argc < 2) return 2;
    std::map<std::string, double> params;
    params["Lx"] = 1.0;
    params["Ly"] = 1.0;
    params["Lz"] = 1.0;
    params["d"] = 0.6;
    params["e"] = 0.0;
    params["M"] = 4;
    params["alpha"] = 1;
    params["boxSize"] = 1;
    params["toPrint"] = 0;
    if (readData(params, argv[1]) != 0) {
        std::printf("readData: cannot open\n");
        return 3;
    }
    for (auto& kv : params) std::printf("map %s %.17g\n", kv.first.c_str(), kv.second);
    std::string names[] = {"Lx", "Ly", "Lz", "d", "e", "M", "alpha", "boxSize", "toPrint"};
    double values[] = {1.0, 1.0, 1.0, 0.6, 0, 4, 1, 1, 0};
    readData(values, names, 9, argv[1]);
    for (int k = 0; k < 9; k++) std::printf("array %s %.17g\n", names[k].c_str(), values[k]);
    std::printf("missing %d\n", readData(params, "no/such/file.txt"));

    const int m = 5, n = 4;
    MatrixOnHost xh(3, m), x0h(3, n), f(3, n), U(3, m), L(3);
    for (int i = 0; i < 3 * m; i++) xh(i) = std::fmod(0.37 * (i + 1), 1.0);
    for (int i = 0; i < 3 * n; i++) x0h(i) = std::fmod(0.61 * (i + 2), 1.0);
    for (int i = 0; i < 3 * n; i++) f(i) = std::sin(1.0 + i);
    L(0) = params["Lx"];
    L(1) = params["Ly"];
    L(2) = params["Lz"];
    const double a = params["alpha"], d = params["d"], e = params["e"];
    const int M = (int)params["M"];
    const int Mg[3] = {32, 32, 32}, Pg[3] = {12, 12, 12};
    try {
        fftBrinkman(U, xh, f, x0h, L, Mg, Pg, 6, 0, e, 1e-6, d, a);
        std::vector<double> U2(3 * m);
        if (pb_fft_brinkman(U2.data(), xh.data(), m, f.data(), x0h.data(), n, L.data(), Mg, Pg, 6, 0, e, 1e-6, d,
                            a) != PB_OK)
            return 4;
        double dmax = 0;
        for (int i = 0; i < 3 * m; i++) dmax = std::fmax(dmax, std::fabs(U(i) - U2[i]));
        std::printf("fftBrinkman diff %.3g norm %.6g\n", dmax, std::fabs(U(0)) + std::fabs(U(1)));
        if (argc > 2 && !std::strcmp(argv[2], "gpu")) {
            double *px, *px0, *pA, *pB;
            cudaMalloc(&px, sizeof(double) * 3 * m);
            cudaMalloc(&px0, sizeof(double) * 3 * n);
            cudaMalloc(&pA, sizeof(double) * 9 * m * n);
            cudaMalloc(&pB, sizeof(double) * 9 * m * n);
            cudaMemcpy(px, xh.data(), sizeof(double) * 3 * m, cudaMemcpyHostToDevice);
            cudaMemcpy(px0, x0h.data(), sizeof(double) * 3 * n, cudaMemcpyHostToDevice);
            cudaMemset(pA, 0, sizeof(double) * 9 * m * n);
            cudaMemset(pB, 0, sizeof(double) * 9 * m * n);
            MatrixOnDevice dA{pA, 3 * m, 3 * n}, dx{px, 3, m}, dx0{px0, 3, n};
            periodicBrinkman(dA, dx, dx0, a, d, e, M, M, L.data());
            if (pb_periodic_brinkman(pB, px, m, px0, n, a, d, e, M, M, L.data(), 256) != PB_OK) return 5;
            std::vector<double> A(9 * m * n), B(9 * m * n);
            cudaMemcpy(A.data(), pA, sizeof(double) * A.size(), cudaMemcpyDeviceToHost);
            cudaMemcpy(B.data(), pB, sizeof(double) * B.size(), cudaMemcpyDeviceToHost);
            double dm = 0, am = 0;
            for (size_t i = 0; i < A.size(); i++) {
                dm = std::fmax(dm, std::fabs(A[i] - B[i]));
                am = std::fmax(am, std::fabs(B[i]));
            }
            std::printf("periodicBrinkman diff %.3g max %.6g\n", dm, am);
            MatrixOnDevice bad{pA, 3 * m, 3 * n + 3};
            try {
                periodicBrinkman(bad, dx, dx0, a, d, e, M, M, L.data());
                std::printf("shape check missing\n");
            } catch (const pbrinkman::error& ex) {
                std::printf("shape error %d\n", ex.code);
            }
            cudaFree(px);
            cudaFree(px0);
            cudaFree(pA);
            cudaFree(pB);
        }
    } catch (const pbrinkman::error& ex) {
        std::printf("error %d %s\n", ex.code, ex.what());
    }
    return 0;
}

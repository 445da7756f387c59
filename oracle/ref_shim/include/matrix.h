/*
 * Stand-in for the reference's missing "../../include/matrix.h".
 *
 * TEST INFRASTRUCTURE ONLY: used by oracle/build_ref.sh to compile the
 * reference's own host code (cuda/periodicBrinkman.h) into oracle/_ref/,
 * which generates the golden fixtures under tests/golden/.
 *
 * The reference header needs, from that library: PI, SPI (= sqrt(pi), the
 * normalisation pi^{3/2} = PI*SPI of the Gaussian blob), the switch radius
 * `eps`, dot() on 3-vectors, host and device column-major matrices
 * (MatrixOnHost / MatrixOnDevice), chooseSize() and warpReduce().  Only the
 * members the reference calls are provided, plus data() (the column-major
 * storage, for include/pbrinkman.hpp's overloads in tests/cxx/).  The
 * reference's kernels are compiled into oracle/_ref/ref_kernels.* and
 * launched by oracle/ref_launch.cpp, never by the fixture generator.
 */
#ifndef PB_REF_SHIM_MATRIX_H
#define PB_REF_SHIM_MATRIX_H
#include <cassert>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>
#include <cuda_runtime.h>

#define PI 3.14159265358979323846264338327950288
#define SPI 1.77245385090551602729816748334114518
/* Switch radius below which the reference uses its r -> 0 limits. */
static constexpr double eps = 1e-12;

__host__ __device__ inline double dot(const double *a, const double *b)
{
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

class MatrixOnHost {
  public:
    MatrixOnHost() : r_(0), c_(0) {}
    MatrixOnHost(int r, int c = 1, double v = 0) : r_(r), c_(c), d_((size_t)r * c, v) {}
    int rows() const { return r_; }
    int columns() const { return c_; }
    double &operator()(int i) { return d_[i]; }
    double operator()(int i) const { return d_[i]; }
    double &operator()(int i, int j) { return d_[(size_t)j * r_ + i]; }
    double operator()(int i, int j) const { return d_[(size_t)j * r_ + i]; }
    operator double *() { return d_.data(); }
    operator const double *() const { return d_.data(); }
    void setElements(double v) { for (auto &x : d_) x = v; }
    double *data() { return d_.data(); }
    const double *data() const { return d_.data(); }

  private:
    int r_, c_;
    std::vector<double> d_;
};

struct MatrixOnDevice {
    double *p;
    int r, c;
    __host__ __device__ int rows() const { return r; }
    __host__ __device__ int columns() const { return c; }
    __host__ __device__ double *data() const { return p; }
    __device__ double &operator()(int i, int j) { return p[(size_t)j * r + i]; }
    __device__ double operator()(int i, int j) const { return p[(size_t)j * r + i]; }
};

inline unsigned chooseSize(unsigned n, unsigned maxBit = 16)
{
    unsigned s = 1;
    while (s < n && s < (1u << maxBit)) s <<= 1;
    return s;
}

#ifdef __CUDACC__  /* device code: only in CUDA translation units (a host C++ caller includes this too) */
__device__ inline void warpReduce(double *U, unsigned tid, unsigned blockSize)
{
    for (unsigned s = 32; s > 0; s >>= 1) {
        if (blockSize > s && tid < s) U[tid] += U[tid + s];
        __syncwarp();
    }
}
#endif
#endif

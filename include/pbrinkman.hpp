/*
 * pbrinkman.hpp -- C++ overloads with the reference's signatures, so that
 * callers written against hoangngan82/periodicBrinkman compile unchanged
 * against this library: periodicBrinkman (cuda/periodicBrinkman.h:432-441),
 * fftBrinkman (cuda/fftBrinkman.h:34-50) and both forms of readData
 * (cuda/periodicBrinkman.cu:44-70, cuda/periodicBrinkman.h:524-554).  Each
 * forwards to the C ABI of pbrinkman.h; a failure throws pbrinkman::error
 * (the reference asserts or carries on silently).
 *
 * The matrices are the caller's own types, as in the reference: the
 * reference's MatrixOnDevice / MatrixOnHost (from its matrix library) or
 * anything with rows(), columns() and column-major storage.  The storage
 * pointer is taken by pbrinkman::matrix_data<M>::get(m), which calls
 * m.data(); specialise it for a matrix type that names it differently.
 *
 * Semantics are the C functions': periodicBrinkman accumulates the real +
 * k-space dense matrix into dA (device memory) with the 1/tau of the
 * reference's host twin; fftBrinkman overwrites U (host memory) with the
 * k-space velocities.  Both synchronise before returning.
 */
#ifndef PBRINKMAN_HPP
#define PBRINKMAN_HPP

#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "pbrinkman.h"

namespace pbrinkman {

// Raised by the overloads below: the PB_ERR_* code and pb_last_error()'s message.
struct error : std::runtime_error {
    int code;
    error(int c, const std::string& msg) : std::runtime_error(msg), code(c) {}
};

inline void check(int rc)
{
    if (rc < 0) throw error(rc, pb_last_error());
}

// Column-major storage of a caller's matrix type (specialise as needed).
template <class M>
struct matrix_data {
    static double* get(const M& m) { return const_cast<double*>(static_cast<const double*>(m.data())); }
};

template <class M>
inline double* data_of(const M& m)
{
    return matrix_data<M>::get(m);
}

}  // namespace pbrinkman

// periodicBrinkman(dA, dx, dx0, a, d, e, M, N, L, maxBlockSize): dA (3m x 3n),
// dx (3 x m), dx0 (3 x n) in DEVICE memory, L three host doubles.
template <class DeviceMatrix>
void periodicBrinkman(DeviceMatrix dA, DeviceMatrix dx, DeviceMatrix dx0, const double& a, const double& d,
                      const double& e, const int& M, const int& N, const double* const L, const int& maxBlockSize = 256)
{
    if (!(dA.rows() == 3 * dx.columns() && dA.columns() == 3 * dx0.columns() && dx.rows() == 3 && dx0.rows() == 3))
        throw pbrinkman::error(PB_ERR_INVALID, "periodicBrinkman: dA must be 3m x 3n for dx 3 x m, dx0 3 x n");
    pbrinkman::check(pb_periodic_brinkman(pbrinkman::data_of(dA), pbrinkman::data_of(dx), dx.columns(),
                                          pbrinkman::data_of(dx0), dx0.columns(), a, d, e, M, N, L, maxBlockSize));
}

// fftBrinkman(U, y, f, xn, L, M, P, m, C, e, tol, d, alpha): HOST matrices
// U, y (3 x m), f, xn (3 x n), L (3 entries); M, P three ints each.
template <class HostMatrix>
void fftBrinkman(HostMatrix& U, const HostMatrix& y, const HostMatrix& f, const HostMatrix& xn, const HostMatrix& L,
                 const int* const M, const int* const P, const int& m, const int& C, const double& e,
                 const double& tol, const double& d, const double& alpha = 1)
{
    if (!(U.rows() == 3 && y.rows() == 3 && f.rows() == 3 && xn.rows() == 3 && U.columns() == y.columns() &&
          f.columns() == xn.columns() && L.rows() * L.columns() >= 3))
        throw pbrinkman::error(PB_ERR_INVALID, "fftBrinkman: U, y 3 x m; f, xn 3 x n; L 3 entries");
    const double* Ld = pbrinkman::data_of(L);
    const double Lv[3] = {Ld[0], Ld[1], Ld[2]};
    pbrinkman::check(pb_fft_brinkman(pbrinkman::data_of(U), pbrinkman::data_of(y), y.columns(),
                                     pbrinkman::data_of(f), pbrinkman::data_of(xn), xn.columns(), Lv, M, P, m, C, e,
                                     tol, d, alpha));
}

// readData(params, fileName, delimiters): the map form.  Returns 0, or 1 if
// the file cannot be read (as the reference does); other errors throw.
inline int readData(std::map<std::string, double>& params, const char* fileName, const char* delimiters = ": ")
{
    std::vector<char> keys(64 * 64);
    std::vector<double> vals(64);
    int n = pb_read_param_file(fileName, delimiters, reinterpret_cast<char(*)[64]>(keys.data()), vals.data(), 64);
    if (n > 64) {
        keys.resize(64 * (size_t)n);
        vals.resize(n);
        n = pb_read_param_file(fileName, delimiters, reinterpret_cast<char(*)[64]>(keys.data()), vals.data(), n);
    }
    if (n < 0) {
        if (n == PB_ERR_INVALID && std::string(pb_last_error()).find("cannot open") != std::string::npos) return 1;
        pbrinkman::check(n);
    }
    for (int k = 0; k < n; k++) params[std::string(&keys[64 * (size_t)k])] = vals[k];
    return 0;
}

// readData(values, names, numel, fileName, delimiters): the array twin.
inline int readData(double* values, const std::string names[], const int& numel, const char* fileName,
                    const char* delimiters = ": ")
{
    std::vector<const char*> p(numel > 0 ? numel : 1);
    for (int k = 0; k < numel; k++) p[k] = names[k].c_str();
    int rc = pb_read_params(fileName, delimiters, p.data(), values, numel);
    if (rc == PB_ERR_INVALID && std::string(pb_last_error()).find("cannot open") != std::string::npos) return 1;
    pbrinkman::check(rc);
    return 0;
}

#endif

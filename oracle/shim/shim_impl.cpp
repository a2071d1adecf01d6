// Test infrastructure (oracle): implementations behind the shim headers.
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>
#include "../cpu_fft.hpp"
#include "cblas.h"
#include "fftw3.h"
#include "lapacke.h"
#include "mpi.h"

// ---- MPI, one rank ---------------------------------------------------------
int MPI_Init(int *, char ***) { return 0; }
int MPI_Finalize() { return 0; }
int MPI_Comm_size(MPI_Comm, int *size) { *size = 1; return 0; }
int MPI_Comm_rank(MPI_Comm, int *rank) { *rank = 0; return 0; }
int MPI_Comm_split(MPI_Comm, int, int, MPI_Comm *out) { *out = 0; return 0; }
int MPI_Barrier(MPI_Comm) { return 0; }
int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
int MPI_Alltoall(const void *send, int scount, MPI_Datatype stype, void *recv, int, MPI_Datatype, MPI_Comm) {
  std::memmove(recv, send, (size_t)scount * (size_t)stype);
  return 0;
}
int MPI_Abort(MPI_Comm, int code) { std::exit(code); }
double MPI_Wtime() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// ---- FFTW plan API on the project FFT ---------------------------------------
struct owt_fftw_plan_s {
  owt_oracle::CpuFft fft;
  fftw_complex *in, *out;
  std::vector<owt_oracle::cplx> work;
};
void *fftw_malloc(size_t n) { return std::malloc(n); }
void fftw_free(void *p) { std::free(p); }
fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out, int sign, unsigned) {
  auto *p = new owt_fftw_plan_s{owt_oracle::CpuFft(n, sign), in, out, std::vector<owt_oracle::cplx>(n)};
  return p;
}
void fftw_execute(const fftw_plan p) {
  auto *in = reinterpret_cast<const owt_oracle::cplx *>(p->in);
  auto *out = reinterpret_cast<owt_oracle::cplx *>(p->out);
  p->fft.exec(in, out, p->work.data());
}
void fftw_destroy_plan(fftw_plan p) { delete p; }

// ---- BLAS / LAPACK subset ----------------------------------------------------
void cblas_dgemm(CBLAS_ORDER, CBLAS_TRANSPOSE, CBLAS_TRANSPOSE, int m, int n, int k, double alpha, const double *a,
                 int lda, const double *b, int ldb, double beta, double *c, int ldc) {
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) {
      double s = 0.0;
      for (int p = 0; p < k; ++p) s += a[i + (size_t)p * lda] * b[p + (size_t)j * ldb];
      c[i + (size_t)j * ldc] = alpha * s + (beta == 0.0 ? 0.0 : beta * c[i + (size_t)j * ldc]);
    }
}

lapack_int LAPACKE_dgetrf(int, lapack_int m, lapack_int n, double *a, lapack_int lda, lapack_int *ipiv) {
  lapack_int info = 0;
  const lapack_int mn = m < n ? m : n;
  for (lapack_int j = 0; j < mn; ++j) {
    lapack_int p = j;
    double best = std::fabs(a[j + (size_t)j * lda]);
    for (lapack_int i = j + 1; i < m; ++i) {
      double v = std::fabs(a[i + (size_t)j * lda]);
      if (v > best) { best = v; p = i; }
    }
    ipiv[j] = p + 1;
    if (a[p + (size_t)j * lda] != 0.0) {
      if (p != j)
        for (lapack_int c = 0; c < n; ++c) std::swap(a[j + (size_t)c * lda], a[p + (size_t)c * lda]);
      const double inv = 1.0 / a[j + (size_t)j * lda];
      for (lapack_int i = j + 1; i < m; ++i) a[i + (size_t)j * lda] *= inv;
    } else if (info == 0) {
      info = j + 1;
    }
    for (lapack_int c = j + 1; c < n; ++c) {
      const double t = a[j + (size_t)c * lda];
      if (t != 0.0)
        for (lapack_int i = j + 1; i < m; ++i) a[i + (size_t)c * lda] -= a[i + (size_t)j * lda] * t;
    }
  }
  return info;
}

template <typename T>
static void getrs_impl(lapack_int n, lapack_int nrhs, const T *a, lapack_int lda, const lapack_int *ipiv, T *b,
                       lapack_int ldb) {
  for (lapack_int r = 0; r < nrhs; ++r) {
    T *x = b + (size_t)r * ldb;
    for (lapack_int i = 0; i < n; ++i) {
      lapack_int p = ipiv[i] - 1;
      if (p != i) std::swap(x[i], x[p]);
    }
    for (lapack_int j = 0; j < n; ++j) {
      const T xj = x[j];
      if (xj != T(0))
        for (lapack_int i = j + 1; i < n; ++i) x[i] -= a[i + (size_t)j * lda] * xj;
    }
    for (lapack_int j = n - 1; j >= 0; --j) {
      if (x[j] != T(0)) {
        x[j] /= a[j + (size_t)j * lda];
        const T xj = x[j];
        for (lapack_int i = 0; i < j; ++i) x[i] -= a[i + (size_t)j * lda] * xj;
      }
    }
  }
}
lapack_int LAPACKE_dgetrs(int, char, lapack_int n, lapack_int nrhs, const double *a, lapack_int lda,
                          const lapack_int *ipiv, double *b, lapack_int ldb) {
  getrs_impl<double>(n, nrhs, a, lda, ipiv, b, ldb);
  return 0;
}
lapack_int LAPACKE_zgetrs(int, char, lapack_int n, lapack_int nrhs, const lapack_complex_double *a, lapack_int lda,
                          const lapack_int *ipiv, lapack_complex_double *b, lapack_int ldb) {
  getrs_impl<lapack_complex_double>(n, nrhs, a, lda, ipiv, b, ldb);
  return 0;
}

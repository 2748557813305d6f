// Benchmark driver with the reference's command line and output:
//
//   ./test <precision> <algorithm> <size> <batch> <repetitions> [out.csv]
//
// precision 0 = float, 1 = double; algorithm = index into the solver table
// (the reference's selector<T>::solvers, Tridiagonal_CUDA/helpers.h:12-65,
// same indices and names; indices from 32 are this library's extensions).
// As the reference driver (Tridiagonal_CUDA/test.cpp:62-155) it builds one
// system with a manufactured solution (x ~ U[-1,1], a, c ~ U[-1,1],
// b = U[0,1] + max(|a_i|+|c_i|, |a_{i+1}|+|c_{i-1}|), d = A x), copies it to
// every batch slot before each repetition (untimed), times each solver call
// with a wall clock (the call synchronises), and reports the 1- and inf-norm
// condition numbers and the mean / RMS / max error of system 0, then appends
// the same CSV row.  The reference draws from MKL's MT19937 (seed 13541532);
// MKL is not available, so this driver uses std::mt19937_64 with that seed.
// The condition numbers come from Hager/Higham 1-norm estimation with a
// pivoted LU of the system (the reference calls LAPACK ?gtcon).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <random>
#include <vector>

#include <cuda_runtime.h>

#include "tridiagonal.h"

namespace {

template <typename T>
struct Solver {
  void (*routine)(T*, T*, T*, T*, int, int);
  const char* name;
  int (*init)(T*, T*, T*, T*, int, int);
  void (*final)();
  int layout;
};

// Extensions (indices 32..): interleaved-layout and pivoted solves through
// the int-returning API, wrapped to the reference's signature.
template <typename T>
void ext_gtsv(T* a, T* b, T* c, T* d, int n, int batch);
template <typename T>
int ext_gtsv_init(T* a, T* b, T* c, T* d, int n, int batch);
void ext_gtsv_final();
template <typename T>
void ext_thomas_interleaved(T* a, T* b, T* c, T* d, int n, int batch);

const Solver<float> kFloat[] = {
    {cuSparse_single, "cuSparse sgtsv", cuSparse_init_single, cuSparse_final, 0},
    {Thomas_single, "Thomas", nullptr, nullptr, 0},
    {CR_single, "CR", CR_init_single, CR_final, 0},
    {PCR5_shmem_single, "shmem PCR-pThomas", nullptr, nullptr, 0},
    {PCR4_shmem_single, "shmem PCR-half-pThomas", nullptr, nullptr, 0},
    {PCR5_reg_single, "reg PCR-pThomas", nullptr, nullptr, 0},
    {PCR4_reg_single, "reg PCR-half-pThomas", nullptr, nullptr, 0},
    {WM5_shmem_single, "shmem WM-pGE", nullptr, nullptr, 0},
    {WM4_shmem_single, "shmem WM-half-pGE", nullptr, nullptr, 0},
    {WM5_reg_single, "reg WM-pGE", nullptr, nullptr, 0},
    {WM4_reg_single, "reg WM-half-pGE", nullptr, nullptr, 0},
    {CR_reg4_single, "reg-4 CR", nullptr, nullptr, 0},
    {CR_reg8_single, "reg-8 CR", nullptr, nullptr, 0},
    {CR_reg16_single, "reg-16 CR", nullptr, nullptr, 0},
    {BPLG_WM, "BPLG WM", nullptr, nullptr, 1},
    {BPLG_LF, "BPLG LF", nullptr, nullptr, 1},
    {BPLG_CR, "BPLG CR", nullptr, nullptr, 1},
    {BPLG_PCR, "BPLG PCR", nullptr, nullptr, 1},
};
const Solver<double> kDouble[] = {
    {cuSparse_double, "cuSparse dgtsv", cuSparse_init_double, cuSparse_final, 0},
    {Thomas_double, "Thomas", nullptr, nullptr, 0},
    {CR_double, "CR", CR_init_double, CR_final, 0},
    {PCR5_shmem_double, "shmem PCR-pThomas", nullptr, nullptr, 0},
    {PCR4_shmem_double, "shmem PCR-half-pThomas", nullptr, nullptr, 0},
    {PCR5_reg_double, "reg PCR-pThomas", nullptr, nullptr, 0},
    {PCR4_reg_double, "reg PCR-half-pThomas", nullptr, nullptr, 0},
    {WM5_shmem_double, "shmem WM-pGE", nullptr, nullptr, 0},
    {WM4_shmem_double, "shmem WM-half-pGE", nullptr, nullptr, 0},
    {WM5_reg_double, "reg WM-pGE", nullptr, nullptr, 0},
    {WM4_reg_double, "reg WM-half-pGE", nullptr, nullptr, 0},
    {CR_reg4_double, "reg-4 CR", nullptr, nullptr, 0},
    {CR_reg8_double, "reg-8 CR", nullptr, nullptr, 0},
    {CR_reg16_double, "reg-16 CR", nullptr, nullptr, 0},
};
constexpr int kExtBase = 32;
const Solver<float> kFloatExt[] = {
    {ext_gtsv<float>, "GB300 pivoted WM-pGE (gtsv)", ext_gtsv_init<float>, ext_gtsv_final, 0},
    {ext_thomas_interleaved<float>, "GB300 Thomas (interleaved layout)", nullptr, nullptr, 2},
};
const Solver<double> kDoubleExt[] = {
    {ext_gtsv<double>, "GB300 pivoted WM-pGE (gtsv)", ext_gtsv_init<double>, ext_gtsv_final, 0},
    {ext_thomas_interleaved<double>, "GB300 Thomas (interleaved layout)", nullptr, nullptr, 2},
};

// The pivoted solve's workspace is allocated by the init hook and freed by
// the final hook, outside the timed calls (the reference's protocol for its
// CR and cuSPARSE rows, Tridiagonal_CUDA/test.cpp:86,107).
void* g_ext_work = nullptr;
size_t g_ext_work_bytes = 0;

template <typename T>
int ext_gtsv_init(T*, T*, T*, T*, int n, int batch) {
  g_ext_work_bytes = tridiag_gtsv_workspace_size(sizeof(T) == 8, 0, n, batch);
  return cudaMalloc(&g_ext_work, g_ext_work_bytes) == cudaSuccess ? 0 : 1;
}

void ext_gtsv_final() {
  cudaFree(g_ext_work);
  g_ext_work = nullptr;
  g_ext_work_bytes = 0;
}

template <typename T>
void ext_gtsv(T* a, T* b, T* c, T* d, int n, int batch) {
  if (!g_ext_work) return;
  if constexpr (sizeof(T) == 8)
    tridiag_gtsv_double(0, a, b, c, d, nullptr, nullptr, g_ext_work, g_ext_work_bytes, n, batch, nullptr);
  else
    tridiag_gtsv_single(0, a, b, c, d, nullptr, nullptr, g_ext_work, g_ext_work_bytes, n, batch, nullptr);
  cudaDeviceSynchronize();
}

template <typename T>
void ext_thomas_interleaved(T* a, T* b, T* c, T* d, int n, int batch) {
  if constexpr (sizeof(T) == 8)
    tridiag_solve_double(TRIDIAG_ALGO_THOMAS, TRIDIAG_LAYOUT_INTERLEAVED, a, b, c, d, n, batch, nullptr);
  else
    tridiag_solve_single(TRIDIAG_ALGO_THOMAS, TRIDIAG_LAYOUT_INTERLEAVED, a, b, c, d, n, batch, nullptr);
  cudaDeviceSynchronize();
}

template <typename T, size_t N>
constexpr int len(const T (&)[N]) {
  return (int)N;
}

template <typename T>
const Solver<T>* pick(int algo);
template <>
const Solver<float>* pick<float>(int algo) {
  if (algo >= 0 && algo < len(kFloat)) return &kFloat[algo];
  if (algo >= kExtBase && algo < kExtBase + len(kFloatExt)) return &kFloatExt[algo - kExtBase];
  return nullptr;
}
template <>
const Solver<double>* pick<double>(int algo) {
  if (algo >= 0 && algo < len(kDouble)) return &kDouble[algo];
  if (algo >= kExtBase && algo < kExtBase + len(kDoubleExt)) return &kDoubleExt[algo - kExtBase];
  return nullptr;
}

// One system with a manufactured solution, the reference generator's
// distribution (Tridiagonal_CUDA/test.cpp:19-38).
template <typename T>
void tridiag_gen(std::vector<T>& a, std::vector<T>& b, std::vector<T>& c, std::vector<T>& d, std::vector<T>& x,
                 int n) {
  std::mt19937_64 rng(13541532);
  std::uniform_real_distribution<double> u11(-1.0, 1.0), u01(0.0, 1.0);
  for (int i = 1; i < n; ++i) a[i] = (T)u11(rng);
  for (int i = 0; i < n - 1; ++i) c[i] = (T)u11(rng);
  for (int i = 0; i < n; ++i) x[i] = (T)u11(rng);
  for (int i = 0; i < n; ++i) b[i] = (T)u01(rng);
  a[0] = 0;
  c[n - 1] = 0;
  auto A = [&](int i) { return i >= 0 && i < n ? std::fabs((double)a[i]) : 0.0; };
  auto C = [&](int i) { return i >= 0 && i < n ? std::fabs((double)c[i]) : 0.0; };
  for (int i = 0; i < n; ++i) {
    b[i] = (T)((double)b[i] + std::max(A(i) + C(i), A(i + 1) + C(i - 1)));
    double s = (double)b[i] * x[i];
    if (i > 0) s += (double)a[i] * x[i - 1];
    if (i < n - 1) s += (double)c[i] * x[i + 1];
    d[i] = (T)s;
  }
}

// Pivoted LU of one system in FP64 (GE with adjacent-row interchange) and
// solves with A or A^T, for the condition estimate.
struct HostLU {
  int n;
  std::vector<double> l, u0, u1, u2;
  std::vector<char> piv;
  template <typename T>
  explicit HostLU(const std::vector<T>& a, const std::vector<T>& b, const std::vector<T>& c)
      : n((int)b.size()), l(n), u0(n), u1(n), u2(n), piv(n) {
    for (int i = 0; i < n; ++i) { u0[i] = b[i]; u1[i] = i + 1 < n ? c[i] : 0; u2[i] = 0; l[i] = 0; piv[i] = 0; }
    for (int i = 0; i + 1 < n; ++i) {
      double sub = a[i + 1];
      if (std::fabs(u0[i]) >= std::fabs(sub)) {
        double m = u0[i] != 0 ? sub / u0[i] : 0;
        u0[i + 1] -= m * u1[i];
        l[i] = m;
      } else {
        double m = u0[i] / sub, t = u0[i + 1];
        u0[i] = sub;
        u0[i + 1] = u1[i] - m * t;
        if (i + 2 < n) { u2[i] = u1[i + 1]; u1[i + 1] = -m * u1[i + 1]; }
        u1[i] = t;
        l[i] = m;
        piv[i] = 1;
      }
    }
  }
  void solve(std::vector<double>& v) const {  // A x = v
    for (int i = 0; i + 1 < n; ++i) {
      if (piv[i]) std::swap(v[i], v[i + 1]);
      v[i + 1] -= l[i] * v[i];
    }
    for (int i = n - 1; i >= 0; --i) {
      double s = v[i];
      if (i + 1 < n) s -= u1[i] * v[i + 1];
      if (i + 2 < n) s -= u2[i] * v[i + 2];
      v[i] = s / u0[i];
    }
  }
  void solve_t(std::vector<double>& v) const {  // A^T x = v
    for (int i = 0; i < n; ++i) {
      double s = v[i];
      if (i >= 1) s -= u1[i - 1] * v[i - 1];
      if (i >= 2) s -= u2[i - 2] * v[i - 2];
      v[i] = s / u0[i];
    }
    for (int i = n - 2; i >= 0; --i) {
      v[i] -= l[i] * v[i + 1];
      if (piv[i]) std::swap(v[i], v[i + 1]);
    }
  }
};

// Hager/Higham estimate of ||A^{-1}||_1 (transpose = false) or
// ||A^{-1}||_inf = ||A^{-T}||_1 (transpose = true).
double inv_norm_est(const HostLU& lu, bool transpose) {
  const int n = lu.n;
  std::vector<double> x(n, 1.0 / n), y, z;
  double est = 0;
  for (int it = 0; it < 5; ++it) {
    y = x;
    transpose ? lu.solve_t(y) : lu.solve(y);
    double e = 0;
    for (double v : y) e += std::fabs(v);
    if (it > 0 && e <= est) break;
    est = e;
    z.assign(n, 0);
    for (int i = 0; i < n; ++i) z[i] = y[i] >= 0 ? 1.0 : -1.0;
    transpose ? lu.solve(z) : lu.solve_t(z);
    int jmax = 0;
    for (int i = 1; i < n; ++i)
      if (std::fabs(z[i]) > std::fabs(z[jmax])) jmax = i;
    x.assign(n, 0);
    x[jmax] = 1;
  }
  return est;
}

void print_algorithms() {
  std::cout << "single-precision algorithms:" << std::endl;
  for (int i = 0; i < len(kFloat); ++i) std::cout << std::setw(3) << i << ": " << kFloat[i].name << std::endl;
  for (int i = 0; i < len(kFloatExt); ++i)
    std::cout << std::setw(3) << kExtBase + i << ": " << kFloatExt[i].name << std::endl;
  std::cout << "double-precision algorithms:" << std::endl;
  for (int i = 0; i < len(kDouble); ++i) std::cout << std::setw(3) << i << ": " << kDouble[i].name << std::endl;
  for (int i = 0; i < len(kDoubleExt); ++i)
    std::cout << std::setw(3) << kExtBase + i << ": " << kDoubleExt[i].name << std::endl;
}

void print_help(const char* argv0) {
  std::cout << "USAGE: " << argv0 << " <precision> <algorithm> <size> <batch> <repetitions> [out file]" << std::endl;
}

template <typename T>
int run(int algo, int size, int batch, int rep, const char* out) {
  const Solver<T>* solver = pick<T>(algo);
  if (!solver) {
    print_algorithms();
    return 1;
  }
  const size_t n = size, slab = n * (size_t)batch;
  std::vector<T> a(n), b(n), c(n), d(n), x(n);
  T* arr = nullptr;
  if (cudaMalloc(&arr, sizeof(T) * 4 * slab) != cudaSuccess) {
    std::cerr << "Not enough GPU memory" << std::endl;
    return 1;
  }
  T *a_batch = arr, *b_batch = arr + slab, *c_batch = arr + 2 * slab, *d_batch = arr + 3 * slab;
  if (solver->init && solver->init(a_batch, b_batch, c_batch, d_batch, size, batch) != 0) {
    std::cerr << "Initialization failed" << std::endl;
    cudaFree(arr);
    return 1;
  }
  std::cout << solver->name << std::endl;
  tridiag_gen<T>(a, b, c, d, x, size);
  // replicated host images of the four arrays in the solver's layout
  std::vector<T> host(4 * slab);
  for (int j = 0; j < batch; ++j)
    for (size_t i = 0; i < n; ++i) {
      const T v[4] = {a[i], b[i], c[i], d[i]};
      for (int k = 0; k < 4; ++k) {
        size_t off;
        if (solver->layout == 1) off = (size_t)j * 4 * n + k * n + i;                 // packed
        else if (solver->layout == 2) off = k * slab + i * (size_t)batch + j;         // interleaved
        else off = k * slab + (size_t)j * n + i;                                      // contiguous
        host[off] = v[k];
      }
    }
  double t_total = 0;
  for (int r = 0; r < rep; ++r) {
    cudaMemcpy(arr, host.data(), sizeof(T) * 4 * slab, cudaMemcpyHostToDevice);
    auto t0 = std::chrono::steady_clock::now();
    if (solver->layout == 1)
      solver->routine(arr, nullptr, nullptr, nullptr, size, batch);
    else
      solver->routine(a_batch, b_batch, c_batch, d_batch, size, batch);
    t_total += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  // system 0 of the result
  std::vector<T> res(n);
  for (size_t i = 0; i < n; ++i) {
    size_t off = solver->layout == 1 ? 3 * n + i : solver->layout == 2 ? 3 * slab + i * (size_t)batch : 3 * slab + i;
    cudaMemcpy(&res[i], arr + off, sizeof(T), cudaMemcpyDeviceToHost);
  }
  cudaFree(arr);
  if (solver->final) solver->final();
  double sum = 0, sq = 0, mx = 0;
  int arg = 0;
  bool nan = false;
  for (size_t i = 0; i < n; ++i) {
    double e = std::fabs((double)res[i] - (double)x[i]);
    if (std::isnan(e)) {
      if (!nan) { nan = true; arg = (int)i; mx = e; }
      sum += e;
      sq += e;
      continue;
    }
    sum += e;
    sq += e * e;
    if (!nan && e >= mx) { mx = e; arg = (int)i; }
  }
  double norm1 = 0, norminf = 0;
  for (size_t i = 0; i < n; ++i) {
    double col = std::fabs((double)b[i]) + (i + 1 < n ? std::fabs((double)a[i + 1]) : 0) + (i > 0 ? std::fabs((double)c[i - 1]) : 0);
    double row = std::fabs((double)a[i]) + std::fabs((double)b[i]) + std::fabs((double)c[i]);
    norm1 = std::max(norm1, col);
    norminf = std::max(norminf, row);
  }
  HostLU lu(a, b, c);
  const double cond1 = norm1 * inv_norm_est(lu, false);
  const double condinf = norminf * inv_norm_est(lu, true);
  const double err1 = sum / n, err2 = std::sqrt(sq / n), errinf = mx;
  const double t = t_total / rep;
  const double throughput = 1e-9 * size * (double)batch * rep / t_total;
  std::cout << std::scientific << "  1-norm condition number: " << cond1 << ", inf-norm condition number: " << condinf
            << std::endl
            << "Cheking error:" << std::endl
            << "Average: " << err1 << std::endl
            << "RMSE:    " << err2 << std::endl
            << "Max:     " << errinf << "  (max position: " << arg << ")" << std::endl
            << std::fixed << "Size:" << std::setw(7) << size << ",   Time: " << std::setprecision(3) << (t * 1e3)
            << " ms,   "
            << "Throughput: " << std::setprecision(6) << throughput << " N/ns" << std::endl
            << std::endl;
  if (out) {
    std::ofstream(out, std::ios_base::app)
        << std::setw(6) << size << ',' << std::setw(8) << batch << ',' << std::setw(25) << solver->name << ','
        << std::fixed << std::setw(15) << std::setprecision(6) << t << ',' << std::setw(15) << std::setprecision(6)
        << throughput << ',' << std::scientific << std::setw(15) << std::setprecision(6) << cond1 << ','
        << std::setw(15) << std::setprecision(6) << condinf << ',' << std::setw(15) << std::setprecision(6) << err1
        << ',' << std::setw(15) << std::setprecision(6) << err2 << ',' << std::setw(15) << std::setprecision(6)
        << errinf << ',' << std::setw(6) << arg << std::endl;
  }
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  std::ios_base::sync_with_stdio(false);
  if (argc < 6) {
    print_help(argv[0]);
    print_algorithms();
    return 1;
  }
  const int prec = std::atoi(argv[1]), algo = std::atoi(argv[2]), size = std::atoi(argv[3]);
  const int batch = std::atoi(argv[4]), rep = std::atoi(argv[5]);
  if (prec < 0 || prec > 1 || algo < 0 || size <= 0 || batch <= 0 || rep <= 0) {
    print_help(argv[0]);
    print_algorithms();
    return 1;
  }
  const char* out = argc > 6 ? argv[6] : nullptr;
  return prec == 0 ? run<float>(algo, size, batch, rep, out) : run<double>(algo, size, batch, rep, out);
}

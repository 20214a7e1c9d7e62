// Host-side input generators for the heat solver (reference initial data and
// the seeded synthetic benchmark configurations).  Pure host C++, no CUDA;
// parallel over k-planes with std::thread so the library does not pull an
// OpenMP runtime into processes that already carry one (PyTorch).
//
// Random numbers are counter based so every cell's value depends only on
// (seed, stream, cell index), not on the thread split:
//   SplitMix64 finaliser (Steele, Lea, Flood, "Fast splittable pseudorandom
//   number generators", OOPSLA 2014) -> 53-bit uniform in [0,1);
//   Box-Muller transform (Box & Muller 1958) -> standard normal.
// Transcendentals (sin, cos, exp, log, sqrt) are the host libm's.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>
#include <algorithm>

#include "heat.h"

namespace {

inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Hash of (seed, stream, index); streams keep kappa, u0 and the bump centre
// independent of one another.
inline uint64_t cell_hash(uint64_t seed, uint64_t stream, uint64_t idx) {
  uint64_t key = splitmix64(seed ^ splitmix64(stream + 0x51ED270B3A6F1C2Dull));
  return splitmix64(key + idx * 0xD1B54A32D192ED03ull);
}

inline double to_unit(uint64_t h) {            // [0,1)
  return (double)(h >> 11) * 0x1.0p-53;
}

inline double uniform01(uint64_t seed, uint64_t stream, uint64_t idx) {
  return to_unit(cell_hash(seed, stream, idx));
}

inline double normal01(uint64_t seed, uint64_t stream, uint64_t idx) {
  // u1 in (0,1] keeps log finite.
  double u1 = ((double)(cell_hash(seed, stream, 2 * idx) >> 11) + 1.0) * 0x1.0p-53;
  double u2 = uniform01(seed, stream, 2 * idx + 1);
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
}

// Run body(k) for k in [0, nz) on up to hardware_concurrency threads.
template <class F>
void parallel_planes(int nz, F body) {
  unsigned nt = std::max(1u, std::thread::hardware_concurrency());
  nt = std::min<unsigned>(nt, (unsigned)nz);
  if (nt <= 1) {
    for (int k = 0; k < nz; ++k) body(k);
    return;
  }
  std::vector<std::thread> th;
  th.reserve(nt);
  for (unsigned t = 0; t < nt; ++t)
    th.emplace_back([=, &body] {
      for (int k = (int)t; k < nz; k += (int)nt) body(k);
    });
  for (auto &x : th) x.join();
}

inline bool on_boundary(int i, int j, int k, int nx, int ny, int nz) {
  return i == 0 || j == 0 || k == 0 || i == nx - 1 || j == ny - 1 || k == nz - 1;
}

double max_of(const double *a, size_t n) {
  double m = -INFINITY;
  for (size_t i = 0; i < n; ++i) m = a[i] > m ? a[i] : m;
  return m;
}

// One pass of a 3x3x3 box filter (mean of the 27 neighbours, indices
// clamped at the faces), separable as three 3-tap means.
void box3_pass(double *a, double *tmp, int nx, int ny, int nz) {
  const size_t sy = (size_t)nx, sz = (size_t)nx * ny;
  // x
  parallel_planes(nz, [&](int k) {
    for (int j = 0; j < ny; ++j) {
      const double *r = a + k * sz + j * sy;
      double *o = tmp + k * sz + j * sy;
      for (int i = 0; i < nx; ++i) {
        int im = i > 0 ? i - 1 : 0, ip = i < nx - 1 ? i + 1 : nx - 1;
        o[i] = (r[im] + r[i] + r[ip]) / 3.0;
      }
    }
  });
  // y
  parallel_planes(nz, [&](int k) {
    for (int j = 0; j < ny; ++j) {
      int jm = j > 0 ? j - 1 : 0, jp = j < ny - 1 ? j + 1 : ny - 1;
      for (int i = 0; i < nx; ++i)
        a[k * sz + j * sy + i] = (tmp[k * sz + jm * sy + i] + tmp[k * sz + j * sy + i] +
                                  tmp[k * sz + jp * sy + i]) / 3.0;
    }
  });
  // z
  parallel_planes(nz, [&](int k) {
    int km = k > 0 ? k - 1 : 0, kp = k < nz - 1 ? k + 1 : nz - 1;
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
        tmp[k * sz + j * sy + i] = (a[km * sz + j * sy + i] + a[k * sz + j * sy + i] +
                                    a[kp * sz + j * sy + i]) / 3.0;
  });
  std::memcpy(a, tmp, sizeof(double) * sz * nz);
}

}  // namespace

extern "C" int heat_inputs_reference(int n, double *kappa, double *rhs, double *u0,
                                     double *h_out, double *dt_out) {
  if (n < 3 || !kappa || !u0) return HEAT_EINVAL;
  // Parameters exactly as heat3D_variable_coeff.c:79-84.
  const double h = 1.0 / (n - 1);
  const double kappa_max = 0.95;
  const double dt = h * h / (12.0 * kappa_max);
  const size_t s = (size_t)n * n;
  // Expressions written as in heat3D_variable_coeff.c:114,121,147 so the
  // host libm sees the same arguments in the same order.
  parallel_planes(n, [&](int k) {
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        size_t idx = k * s + (size_t)j * n + i;
        if (rhs) rhs[idx] = dt * (1.0 + cos(M_PI * i * h) * cos(M_PI * j * h) * cos(M_PI * k * h));
        kappa[idx] = 0.5 + 0.45 * sin(M_PI * i * h) * sin(M_PI * j * h) * sin(M_PI * k * h);
        u0[idx] = on_boundary(i, j, k, n, n, n)
                      ? 0.0
                      : sin(M_PI * i * h) * sin(M_PI * j * h) * sin(M_PI * k * h);
      }
  });
  if (h_out) *h_out = h;
  if (dt_out) *dt_out = dt;
  return HEAT_OK;
}

extern "C" int heat_inputs_config(int cfg, uint64_t seed, int nx, int ny, int nz,
                                  double *kappa, double *u0, double *h_out,
                                  double *dt_out) {
  if (nx < 3 || ny < 3 || nz < 3 || !kappa || !u0 || cfg < 0 || cfg > 4) return HEAT_EINVAL;
  const int nmax = std::max(nx, std::max(ny, nz));
  const double h = 1.0 / (nmax - 1);
  const size_t sy = (size_t)nx, sz = (size_t)nx * ny, total = sz * nz;
  enum { S_KAPPA = 1, S_U0 = 2, S_CENTRE = 3 };

  if (cfg == 1) {
    const double x0 = 0.3 + 0.4 * uniform01(seed, S_CENTRE, 0);
    const double y0 = 0.3 + 0.4 * uniform01(seed, S_CENTRE, 1);
    const double z0 = 0.3 + 0.4 * uniform01(seed, S_CENTRE, 2);
    const double two_sig2 = 2.0 * 0.05 * 0.05;
    parallel_planes(nz, [&](int k) {
      const double z = k * h;
      for (int j = 0; j < ny; ++j) {
        const double y = j * h;
        for (int i = 0; i < nx; ++i) {
          const double x = i * h;
          size_t idx = k * sz + j * sy + i;
          kappa[idx] = 1.0 + 0.9 * std::sin(2.0 * M_PI * x) * std::sin(4.0 * M_PI * y) *
                                 std::cos(2.0 * M_PI * z);
          double r2 = (x - x0) * (x - x0) + (y - y0) * (y - y0) + (z - z0) * (z - z0);
          u0[idx] = on_boundary(i, j, k, nx, ny, nz) ? 0.0 : std::exp(-r2 / two_sig2);
        }
      }
    });
  } else {
    const double sigma = (cfg == 2) ? 1.0 : 0.5;
    parallel_planes(nz, [&](int k) {
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          size_t idx = k * sz + j * sy + i;
          kappa[idx] = std::exp(sigma * normal01(seed, S_KAPPA, idx));
          u0[idx] = on_boundary(i, j, k, nx, ny, nz) ? 0.0 : uniform01(seed, S_U0, idx);
        }
    });
    if (cfg == 2) {
      std::vector<double> tmp;
      try {
        tmp.resize(total);
      } catch (...) {
        return HEAT_ENOMEM;
      }
      for (int p = 0; p < 3; ++p) box3_pass(kappa, tmp.data(), nx, ny, nz);
    }
  }
  const double kmax = max_of(kappa, total);
  if (h_out) *h_out = h;
  if (dt_out) *dt_out = 0.9 * h * h / (6.0 * kmax);
  return HEAT_OK;
}

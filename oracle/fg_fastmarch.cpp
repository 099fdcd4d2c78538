// Accuracy harness (test infrastructure, not part of the product): arrival
// times of the eikonal equation |grad T| = 1 / speed from seed cells, by the
// fast marching solver the reference vendors (dependency/fmm, header-only,
// thinks::fast_marching_method, MIT licence), used the way the reference's
// fast-marching transforms use it (FastGeodis/geodis_fastmarch.cpp:40-57:
// HighAccuracyVaryingSpeedEikonalSolver + SignedArrivalTime, boundary times 0).
//
// The header is compiled from where it lies (the reference tree, or its staged
// copy); the speed field is computed by the caller (oracle/fastmarch.py).
// Arrays are C-ordered with the last axis fastest; the solver's first grid
// axis is its fastest, so the axes are handed over in reverse order.

#include <array>
#include <cstdint>
#include <exception>
#include <string>
#include <vector>

#include "thinks/fast_marching_method/fast_marching_method.hpp"

namespace fmm = thinks::fast_marching_method;

namespace {

std::string g_err;

template <std::size_t N>
int solve(const int *dims, const float *speed, const unsigned char *seed, const float *spacing, float *out) {
  // dims / spacing: slowest axis first (C order); the solver wants fastest first
  std::array<std::size_t, N> size;
  std::array<float, N> sp;
  std::size_t n = 1;
  for (std::size_t k = 0; k < N; k++) {
    size[k] = static_cast<std::size_t>(dims[N - 1 - k]);
    sp[k] = spacing[N - 1 - k];
    n *= size[k];
  }
  std::vector<float> speed_buf(speed, speed + n);
  std::vector<std::array<std::int32_t, N>> seeds;
  std::vector<float> times;
  for (std::size_t i = 0; i < n; i++) {
    if (!seed[i]) continue;
    std::array<std::int32_t, N> idx;
    std::size_t r = i;
    for (std::size_t k = 0; k < N; k++) {  // fastest axis first
      idx[k] = static_cast<std::int32_t>(r % size[k]);
      r /= size[k];
    }
    seeds.push_back(idx);
    times.push_back(0.0f);
  }
  try {
    auto solver = fmm::HighAccuracyVaryingSpeedEikonalSolver<float, N>(sp, size, speed_buf);
    std::vector<float> t = fmm::SignedArrivalTime(size, seeds, times, solver);
    for (std::size_t i = 0; i < n; i++) out[i] = t[i];
  } catch (const std::exception &e) {
    g_err = e.what();
    return -1;
  }
  return 0;
}

}  // namespace

extern "C" {

// ndim 2 or 3; dims, spacing: ndim values, slowest axis first; speed, seed,
// out: prod(dims) values in C order (seed: nonzero = a boundary cell, time 0).
int fgo_fastmarch(int ndim, const int *dims, const float *speed, const unsigned char *seed, const float *spacing,
                  float *out) {
  if (ndim == 2) return solve<2>(dims, speed, seed, spacing, out);
  if (ndim == 3) return solve<3>(dims, speed, seed, spacing, out);
  g_err = "ndim must be 2 or 3";
  return -1;
}

const char *fgo_fastmarch_error(void) { return g_err.c_str(); }

}  // extern "C"

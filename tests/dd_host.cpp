// Host build of the float-float arithmetic (nalu-wind_gb300/csrc/dd.h) for
// the CPU error-bound tests (tests/test_dd_arith.py). Results are returned
// as (hi, lo) float pairs.
#include <cstdint>

#include "dd.h"

using nw::dd;

extern "C" {

void dd_split(int64_t n, const double* x, float* hi, float* lo) {
  for (int64_t i = 0; i < n; ++i) {
    const dd v = nw::dd_from_double(x[i]);
    hi[i] = v.hi;
    lo[i] = v.lo;
  }
}

void dd_back(int64_t n, const float* hi, const float* lo, double* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = nw::dd_to_double(dd{hi[i], lo[i]});
}

void dd_back_int(int64_t n, const float* hi, const float* lo, double* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = nw::dd_to_double_int(dd{hi[i], lo[i]});
}

void dd_widen(int64_t n, const float* f, double* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = nw::widen(f[i]);
}

// op 0: a + b, 1: a - b, 2: a * b, 3: 1 / a, 4: a * float(b.hi)
void dd_binop(int op, int64_t n, const float* ah, const float* al, const float* bh,
              const float* bl, float* rh, float* rl) {
  for (int64_t i = 0; i < n; ++i) {
    const dd a{ah[i], al[i]}, b{bh[i], bl[i]};
    dd r{};
    switch (op) {
      case 0: r = a + b; break;
      case 1: r = a - b; break;
      case 2: r = a * b; break;
      case 3: r = nw::dd_rcp(a); break;
      default: r = a * b.hi; break;
    }
    rh[i] = r.hi;
    rl[i] = r.lo;
  }
}

// sums of k consecutive pairs with the deferred-renormalisation
// accumulator (dd_acc), one result per group
void dd_accsum(int64_t groups, int k, const float* hi, const float* lo, float* rh, float* rl) {
  for (int64_t g = 0; g < groups; ++g) {
    nw::dd_acc a;
    for (int j = 0; j < k; ++j) nw::acc_add(a, dd{hi[g * k + j], lo[g * k + j]});
    const dd r = nw::acc_value(a);
    rh[g] = r.hi;
    rl[g] = r.lo;
  }
}

}  // extern "C"

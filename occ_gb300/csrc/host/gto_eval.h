// Contracted Gaussian shell evaluation shared by the host set-up (shell decay
// radii) and the device collocation kernels.  Cartesian monomials in CCA order
// (xx, xy, xz, yy, yz, zz, ...); pure shells are combined into real solid
// harmonics m = -l..l by a transform table; the result is scaled by OCC's
// common_fac (src/gto/gto.cpp:7-16).  This reproduces what OCC obtains from
// gau2grid (src/gto/gto.cpp:212-287).
#pragma once
#ifdef __CUDACC__
#define OCCX_HD __host__ __device__ __forceinline__
#define OCCX_CHD __host__ __device__ constexpr
#else
#define OCCX_HD inline
#define OCCX_CHD constexpr
#endif

namespace occx {

constexpr int kMaxL = 4;
OCCX_CHD int ncart_of(int l) { return (l + 1) * (l + 2) / 2; }
// Offset of the (2l+1) x ncart(l) transform block of angular momentum l.
OCCX_CHD int sph_offset(int l) {
  int o = 0;
  for (int k = 0; k < l; k++)
    o += (2 * k + 1) * ncart_of(k);
  return o;
}
constexpr int kSphTableSize = sph_offset(kMaxL + 1);

// Cartesian monomial values and gradients for angular momentum l at
// displacement (x, y, z) with radial part R and dR = (1/r) dR/dr, i.e. the
// gradient of R is (x, y, z) * dR.  Outputs have ncart(l) entries.
template <typename T>
OCCX_HD void cart_eval(int l, T x, T y, T z, T R, T dR, T *v, T *gx, T *gy, T *gz) {
  // powers x^0..x^(l+1)
  T px[kMaxL + 2], py[kMaxL + 2], pz[kMaxL + 2];
  px[0] = py[0] = pz[0] = T(1);
  for (int i = 1; i <= l + 1; i++) {
    px[i] = px[i - 1] * x;
    py[i] = py[i - 1] * y;
    pz[i] = pz[i - 1] * z;
  }
  int i = 0;
  for (int a = l; a >= 0; a--) {
    for (int b = l - a; b >= 0; b--) {
      int c = l - a - b;
      T mono = px[a] * py[b] * pz[c];
      v[i] = mono * R;
      if (gx) {
        T dxm = a > 0 ? T(a) * px[a - 1] * py[b] * pz[c] : T(0);
        T dym = b > 0 ? T(b) * px[a] * py[b - 1] * pz[c] : T(0);
        T dzm = c > 0 ? T(c) * px[a] * py[b] * pz[c - 1] : T(0);
        gx[i] = dxm * R + mono * x * dR;
        gy[i] = dym * R + mono * y * dR;
        gz[i] = dzm * R + mono * z * dR;
      }
      i++;
    }
  }
}

// Compile-time angular momentum variant (the device kernels dispatch on l so
// that the monomial arrays stay in registers).
template <int L, typename T>
OCCX_HD void cart_eval_l(T x, T y, T z, T R, T dR, T *v, T *gx, T *gy, T *gz) {
  T px[L + 2], py[L + 2], pz[L + 2];
  px[0] = py[0] = pz[0] = T(1);
#pragma unroll
  for (int i = 1; i <= L + 1; i++) {
    px[i] = px[i - 1] * x;
    py[i] = py[i - 1] * y;
    pz[i] = pz[i - 1] * z;
  }
  int i = 0;
#pragma unroll
  for (int a = L; a >= 0; a--) {
#pragma unroll
    for (int b = L - a; b >= 0; b--) {
      const int c = L - a - b;
      T mono = px[a] * py[b] * pz[c];
      v[i] = mono * R;
      if (gx) {
        T dxm = a > 0 ? T(a) * px[a > 0 ? a - 1 : 0] * py[b] * pz[c] : T(0);
        T dym = b > 0 ? T(b) * px[a] * py[b > 0 ? b - 1 : 0] * pz[c] : T(0);
        T dzm = c > 0 ? T(c) * px[a] * py[b] * pz[c > 0 ? c - 1 : 0] : T(0);
        gx[i] = dxm * R + mono * x * dR;
        gy[i] = dym * R + mono * y * dR;
        gz[i] = dzm * R + mono * z * dR;
      }
      i++;
    }
  }
}

} // namespace occx

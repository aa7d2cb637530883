// Forward-mode dual numbers for the adjoint kernels.
//
// Dual<R, W> carries a value and W directional derivatives.  The adjoint
// (reverse-mode) kernels use it locally: one interaction's inputs are seeded
// W at a time, the interaction is evaluated once in Dual arithmetic, and the
// resulting Jacobian columns are contracted with the output adjoint; the
// contribution is then scattered into the global adjoint arrays.  Branches
// (cut-offs, clamps, the sign choices of the Euler angles) are taken on the
// value, so every derivative is that of the branch the forward pass took.
//
// The header compiles as CUDA (host + device) and as plain C++.
#pragma once
#include <math.h>

#if defined(__CUDACC__)
#define ADJ_HD __host__ __device__ inline
#else
#define ADJ_HD inline
#endif

namespace adj {

ADJ_HD float vsqrt(float x) { return sqrtf(x); }
ADJ_HD double vsqrt(double x) { return sqrt(x); }
ADJ_HD float vsin(float x) { return sinf(x); }
ADJ_HD double vsin(double x) { return sin(x); }
ADJ_HD float vcos(float x) { return cosf(x); }
ADJ_HD double vcos(double x) { return cos(x); }
ADJ_HD float vtan(float x) { return tanf(x); }
ADJ_HD double vtan(double x) { return tan(x); }
ADJ_HD float vacos(float x) { return acosf(x); }
ADJ_HD double vacos(double x) { return acos(x); }
ADJ_HD float vexp(float x) { return expf(x); }
ADJ_HD double vexp(double x) { return exp(x); }
ADJ_HD float val(float x) { return x; }
ADJ_HD double val(double x) { return x; }
// x^k for a small non-negative integer k (square-and-multiply)
template <class T>
ADJ_HD T ipow(T x, int k) {
  T r(1.0);
  T b = x;
  while (k > 0) {
    if (k & 1) r = r * b;
    k >>= 1;
    if (k) b = b * b;
  }
  return r;
}

// Dual<R, W, G>: value of type R, derivatives of type G (G = R by
// default).  G = float with R = double keeps every value - and every
// elementary function's derivative, evaluated at the value - in FP64, while
// the W directional derivatives propagate in FP32: the FP64 pipe does the
// primal once, the FP32 pipe the W-fold tangent arithmetic.
template <class R, int W, class G = R>
struct Dual {
  using real = R;
  R v;
  G d[W];
  ADJ_HD Dual() {}
  template <class S>
  ADJ_HD explicit Dual(S x) : v(R(x)) {
    for (int i = 0; i < W; i++) d[i] = G(0);
  }
};

template <class T>
struct RealOf {
  using type = T;
};
template <class R, int W, class G>
struct RealOf<Dual<R, W, G>> {
  using type = R;
};

template <class R, int W, class G>
ADJ_HD R val(const Dual<R, W, G>& a) {
  return a.v;
}

#define ADJ_DUAL template <class R, int W, class G> ADJ_HD Dual<R, W, G>
ADJ_DUAL operator+(const Dual<R, W, G>& a, const Dual<R, W, G>& b) {
  Dual<R, W, G> o;
  o.v = a.v + b.v;
  for (int i = 0; i < W; i++) o.d[i] = a.d[i] + b.d[i];
  return o;
}
ADJ_DUAL operator-(const Dual<R, W, G>& a, const Dual<R, W, G>& b) {
  Dual<R, W, G> o;
  o.v = a.v - b.v;
  for (int i = 0; i < W; i++) o.d[i] = a.d[i] - b.d[i];
  return o;
}
ADJ_DUAL operator-(const Dual<R, W, G>& a) {
  Dual<R, W, G> o;
  o.v = -a.v;
  for (int i = 0; i < W; i++) o.d[i] = -a.d[i];
  return o;
}
ADJ_DUAL operator*(const Dual<R, W, G>& a, const Dual<R, W, G>& b) {
  Dual<R, W, G> o;
  o.v = a.v * b.v;
  const G av = G(a.v), bv = G(b.v);
  for (int i = 0; i < W; i++) o.d[i] = a.d[i] * bv + av * b.d[i];
  return o;
}
ADJ_DUAL operator/(const Dual<R, W, G>& a, const Dual<R, W, G>& b) {
  Dual<R, W, G> o;
  const R ib = R(1) / b.v;
  o.v = a.v * ib;
  const G ov = G(o.v), ibg = G(ib);
  for (int i = 0; i < W; i++) o.d[i] = (a.d[i] - ov * b.d[i]) * ibg;
  return o;
}
ADJ_DUAL operator+(const Dual<R, W, G>& a, typename Dual<R, W, G>::real b) {
  Dual<R, W, G> o = a;
  o.v = a.v + b;
  return o;
}
ADJ_DUAL operator+(typename Dual<R, W, G>::real b, const Dual<R, W, G>& a) { return a + b; }
ADJ_DUAL operator-(const Dual<R, W, G>& a, typename Dual<R, W, G>::real b) {
  Dual<R, W, G> o = a;
  o.v = a.v - b;
  return o;
}
ADJ_DUAL operator-(typename Dual<R, W, G>::real b, const Dual<R, W, G>& a) {
  Dual<R, W, G> o = -a;
  o.v = b - a.v;
  return o;
}
ADJ_DUAL operator*(const Dual<R, W, G>& a, typename Dual<R, W, G>::real b) {
  Dual<R, W, G> o;
  o.v = a.v * b;
  const G bg = G(b);
  for (int i = 0; i < W; i++) o.d[i] = a.d[i] * bg;
  return o;
}
ADJ_DUAL operator*(typename Dual<R, W, G>::real b, const Dual<R, W, G>& a) { return a * b; }
ADJ_DUAL operator/(const Dual<R, W, G>& a, typename Dual<R, W, G>::real b) {
  Dual<R, W, G> o;
  o.v = a.v / b;
  const G bg = G(b);
  for (int i = 0; i < W; i++) o.d[i] = a.d[i] / bg;
  return o;
}
ADJ_DUAL operator/(typename Dual<R, W, G>::real b, const Dual<R, W, G>& a) {
  Dual<R, W, G> o;
  o.v = b / a.v;
  const G k = G(-o.v / a.v);
  for (int i = 0; i < W; i++) o.d[i] = k * a.d[i];
  return o;
}

// elementary functions: f(a) with f'(a) applied to every derivative
template <class R, int W, class G>
ADJ_HD Dual<R, W, G> chain_(const Dual<R, W, G>& a, R fv, R fd) {
  Dual<R, W, G> o;
  o.v = fv;
  const G f = G(fd);
  for (int i = 0; i < W; i++) o.d[i] = f * a.d[i];
  return o;
}
ADJ_DUAL vsqrt(const Dual<R, W, G>& a) {
  const R s = vsqrt(a.v);
  return chain_(a, s, R(0.5) / s);
}
ADJ_DUAL vsin(const Dual<R, W, G>& a) { return chain_(a, vsin(a.v), vcos(a.v)); }
ADJ_DUAL vcos(const Dual<R, W, G>& a) { return chain_(a, vcos(a.v), -vsin(a.v)); }
ADJ_DUAL vtan(const Dual<R, W, G>& a) {
  const R t = vtan(a.v);
  return chain_(a, t, R(1) + t * t);
}
ADJ_DUAL vacos(const Dual<R, W, G>& a) { return chain_(a, vacos(a.v), -R(1) / vsqrt(R(1) - a.v * a.v)); }
ADJ_DUAL vexp(const Dual<R, W, G>& a) {
  const R e = vexp(a.v);
  return chain_(a, e, e);
}
#undef ADJ_DUAL

// ---------------------------------------------------------------- 3-vectors
template <class T>
ADJ_HD T dot3(const T* u, const T* v) {
  return u[0] * v[0] + u[1] * v[1] + u[2] * v[2];
}
template <class T>
ADJ_HD void cross3(const T* u, const T* v, T* w) {
  T w0 = u[1] * v[2] - u[2] * v[1];
  T w1 = u[2] * v[0] - u[0] * v[2];
  T w2 = u[0] * v[1] - u[1] * v[0];
  w[0] = w0;
  w[1] = w1;
  w[2] = w2;
}
template <class T>
ADJ_HD T norm3(const T* v) {
  return vsqrt(dot3(v, v));
}

// The vector-Jacobian product of y = f(x) (NIN inputs, NOUT outputs) for
// the W inputs [chunk*W, chunk*W + W): xbar[j] = sum_o ybar[o] dy_o/dx_{chunk*W+j}.
// f is called as f(const Dual* x, Dual* y).
#if defined(__CUDACC__)
#pragma nv_exec_check_disable
#endif
template <int W, int NIN, int NOUT, class G, class R, class F>
ADJ_HD void vjp_chunk_g(const F& f, const R* x, const R* ybar, int chunk, R* xbar) {
  using D = Dual<R, W, G>;
  D xd[NIN];
  D yd[NOUT];
  for (int k = 0; k < NIN; k++) {
    xd[k] = D(x[k]);
    const int j = k - chunk * W;
    if (j >= 0 && j < W) xd[k].d[j] = G(1);
  }
  for (int o = 0; o < NOUT; o++) yd[o] = D(0.0);
  f(xd, yd);
  for (int j = 0; j < W; j++) {
    R s = R(0);
    for (int o = 0; o < NOUT; o++) s += ybar[o] * R(yd[o].d[j]);
    xbar[j] = s;
  }
}
// derivatives in the value's own type
#if defined(__CUDACC__)
#pragma nv_exec_check_disable
#endif
template <int W, int NIN, int NOUT, class R, class F>
ADJ_HD void vjp_chunk(const F& f, const R* x, const R* ybar, int chunk, R* xbar) {
  vjp_chunk_g<W, NIN, NOUT, R>(f, x, ybar, chunk, xbar);
}

}  // namespace adj

// solvers.cuh -- CG, BiCGStab and GMRES with every reduction, scalar
// recurrence and convergence test on the device.  Each solver_<method>_<type>.cu
// translation unit instantiates one of them for one value type, so the six
// compile in parallel.
//
// Each solver is a fixed sequence of fused kernels per iteration; scalars
// live in a device state struct written by the last block of the kernel that
// completes the reduction, and read by the next kernel.  The iterations loop
// on the device (run_iterations); small systems run in one cluster launch.
#pragma once
#include <algorithm>
#include <cmath>

#include <cooperative_groups.h>

#include "formats.hpp"
#include "vecpass.cuh"

namespace cg = cooperative_groups;

namespace vclgb {

template <typename T>
struct St {
  T rr, ApAp, pAp, alpha, beta, omega;
  T nrhs, nrhs2, ip, vnorm2;
  T Ap_r0, s_s, r_r0, resnorm;
  double tol, abs_tol, error;
  unsigned iters, max_iters, last_restart, max_before_restart;
  int done;
  int restart;
  int restart_skip;  // done || !restart (skip flag for the restart kernels)
};

template <typename T>
__device__ __forceinline__ bool finite_(T v) { return isfinite(v); }

struct NoScal {};

// ===========================================================================
// pipelined CG (cg.hpp:128-187; fused kernels as in
// host_based/iterative_operations.hpp:52-105 and 378-416)
// ===========================================================================
template <typename T>
struct CgInit {
  static constexpr int NDOT = 1;
  const T *b; T *x, *r, *p; St<T> *st;
  __device__ bool skip() const { return false; }
  __device__ NoScal load() const { return {}; }
  __device__ void apply(size_t i, NoScal, T (&d)[1]) const {
    T bi = b[i];
    x[i] = T(0); r[i] = bi; p[i] = bi;
    d[0] += bi * bi;
  }
  __device__ void finalize(const T (&s)[1]) const {
    T nrm = sqrt(s[0]);
    st->nrhs2 = nrm * nrm;  // norm_2(residual)^2 as cg.hpp:149
    st->rr = st->nrhs2;
    st->iters = 0;
    st->error = 0;
    st->done = (st->nrhs2 <= T(st->abs_tol * st->abs_tol)) ? kConverged : kRunning;
  }
};

template <typename T>
struct EpiCgFirst {  // Ap = A p; alpha = rr/<p,Ap>; beta = (alpha^2 ||Ap||^2 - rr)/rr
  static constexpr int NDOT = 2;
  T *Ap; const T *p; St<T> *st;
  struct Pre { T p; };
  __device__ bool skip() const { return st->done != kRunning; }
  __device__ Pre pre(uint32_t r) const { return {p[r]}; }
  __device__ void row(uint32_t r, T acc, const Pre &v, T (&d)[2]) const {
    Ap[r] = acc;
    d[0] += acc * acc;
    d[1] += v.p * acc;
  }
  __device__ void finalize(const T (&s)[2]) const {
    T rr = st->rr;
    T alpha = rr / s[1];
    T nap = sqrt(s[0]);
    st->alpha = alpha;
    st->beta = (alpha * alpha * nap * nap - rr) / rr;
    if (st->max_iters == 0) {
      st->done = kMaxIters;
      st->error = sqrt(fabs((double)rr) / (double)st->nrhs2);
    }
  }
};

template <typename T>
struct CgUpdate {  // x += a p; r -= a Ap; p = r + b p; <r,r>
  static constexpr int NDOT = 1;
  T *x, *p, *r; const T *Ap; St<T> *st;
  struct S { T a, b; };
  __device__ bool skip() const { return st->done != kRunning; }
  __device__ S load() const { return {st->alpha, st->beta}; }
  __device__ void apply(size_t i, S s, T (&d)[1]) const {
    T vp = p[i], vr = r[i];
    x[i] += s.a * vp;
    vr -= s.a * Ap[i];
    vp = vr + s.b * vp;
    d[0] += vr * vr;
    p[i] = vp;
    r[i] = vr;
  }
  __device__ void finalize(const T (&s)[1]) const { st->rr = s[0]; }
};

template <typename T>
struct EpiCg {  // Ap = A p, <Ap,Ap>, <p,Ap>; convergence test; next alpha/beta
  static constexpr int NDOT = 2;
  T *Ap; const T *p; St<T> *st;
  struct Pre { T p; };
  __device__ bool skip() const { return st->done != kRunning; }
  __device__ Pre pre(uint32_t r) const { return {p[r]}; }
  __device__ void row(uint32_t r, T acc, const Pre &v, T (&d)[2]) const {
    Ap[r] = acc;
    d[0] += acc * acc;
    d[1] += v.p * acc;
  }
  __device__ void finalize(const T (&s)[2]) const {
    st->iters += 1;
    T rr = st->rr;
    double ratio = fabs((double)rr / (double)st->nrhs2);
    if (ratio < st->tol * st->tol || fabs((double)rr) < st->abs_tol * st->abs_tol) {
      st->done = kConverged;
      st->error = sqrt(fabs((double)rr) / (double)st->nrhs2);
      return;
    }
    T alpha = rr / s[1];
    T beta = (alpha * alpha * s[0] - rr) / rr;
    st->alpha = alpha;
    st->beta = beta;
    st->error = sqrt(fabs((double)rr) / (double)st->nrhs2);
    if (!finite_(alpha) || !finite_(beta)) st->done = kBreakdown;
    else if (st->iters >= st->max_iters) st->done = kMaxIters;
  }
};

// ===========================================================================
// preconditioned CG (cg.hpp:257-322)
// ===========================================================================
// JAC: Jacobi fused (z = r * (1/d), the reciprocal formed once with the
// preconditioner); otherwise the preconditioner runs between kernels.  A compile-time choice: a runtime flag let the compiler predicate
// the FP64 division sequence into the non-Jacobi path.
template <typename T, bool JAC>
struct PcgInit {  // x = 0; r = b; z = b/d (or z = b); p = z; <r,z>
  static constexpr int NDOT = 1;
  static constexpr bool jacobi = JAC;
  const T *b, *dg; T *x, *r, *z, *p; St<T> *st;
  __device__ bool skip() const { return false; }
  __device__ NoScal load() const { return {}; }
  __device__ void apply(size_t i, NoScal, T (&d)[1]) const {
    T bi = b[i];
    x[i] = T(0); r[i] = bi;
    if (jacobi) {
      T zi = bi * dg[i];
      p[i] = zi;
      d[0] += bi * zi;
    } else {
      z[i] = bi;
    }
  }
  __device__ void finalize(const T (&s)[1]) const {
    st->iters = 0;
    st->error = 0;
    st->ip = s[0];
    st->nrhs2 = s[0];
    st->done = (fabs((double)s[0]) <= st->abs_tol * st->abs_tol) ? kConverged : kRunning;
    if (st->done == kRunning && st->max_iters == 0) st->done = kMaxIters;
  }
};

template <typename T>
struct PcgInitFinish {  // generic preconditioner: p = z; <r,z>
  static constexpr int NDOT = 1;
  const T *r, *z; T *p; St<T> *st;
  __device__ bool skip() const { return false; }
  __device__ NoScal load() const { return {}; }
  __device__ void apply(size_t i, NoScal, T (&d)[1]) const {
    T zi = z[i];
    p[i] = zi;
    d[0] += r[i] * zi;
  }
  __device__ void finalize(const T (&s)[1]) const {
    st->iters = 0;
    st->error = 0;
    st->ip = s[0];
    st->nrhs2 = s[0];
    st->done = (fabs((double)s[0]) <= st->abs_tol * st->abs_tol) ? kConverged : kRunning;
    if (st->done == kRunning && st->max_iters == 0) st->done = kMaxIters;
  }
};

template <typename T>
struct EpiPcg {  // tmp = A p; alpha = ip / <tmp,p>
  static constexpr int NDOT = 1;
  T *tmp; const T *p; St<T> *st;
  struct Pre { T p; };
  __device__ bool skip() const { return st->done != kRunning; }
  __device__ Pre pre(uint32_t r) const { return {p[r]}; }
  __device__ void row(uint32_t r, T acc, const Pre &v, T (&d)[1]) const {
    tmp[r] = acc;
    d[0] += acc * v.p;
  }
  __device__ void finalize(const T (&s)[1]) const {
    st->iters += 1;
    st->alpha = st->ip / s[0];
    if (!finite_(st->alpha)) st->done = kBreakdown;
  }
};

template <typename T>
__device__ __forceinline__ void pcg_check(St<T> *st, T new_ip) {
  double ratio = (double)new_ip / (double)st->nrhs2;
  st->error = sqrt(fabs(ratio));
  if (fabs(ratio) < st->tol * st->tol || fabs((double)new_ip) < st->abs_tol * st->abs_tol) {
    st->done = kConverged;
    return;
  }
  st->beta = new_ip / st->ip;
  st->ip = new_ip;
  if (!finite_(st->beta)) st->done = kBreakdown;
  else if (st->iters >= st->max_iters) st->done = kMaxIters;
}

// Jacobi: z = r / d is formed once per iteration here (as r times the
// reciprocal diagonal) and stored; PcgP reads it back (the write of z replaces
// PcgP's reads of r and d).
template <typename T, bool JAC>
struct PcgUpdate {  // x += a p; r -= a tmp; z = r/d, <r,z> (Jacobi) / z = r (generic)
  static constexpr int NDOT = JAC ? 1 : 0;
  static constexpr bool jacobi = JAC;
  T *x, *r, *z; const T *p, *tmp, *dg; St<T> *st;
  struct S { T a; };
  __device__ bool skip() const { return st->done != kRunning; }
  __device__ S load() const { return {st->alpha}; }
  __device__ void apply(size_t i, S s, T (&d)[1]) const {
    T vp = p[i];
    x[i] += s.a * vp;
    T vr = r[i] - s.a * tmp[i];
    r[i] = vr;
    if constexpr (JAC) {
      const T zi = vr * dg[i];
      z[i] = zi;
      d[0] += vr * zi;
    } else {
      z[i] = vr;
    }
  }
  __device__ void finalize(const T (&s)[1]) const {
    if constexpr (JAC) pcg_check(st, s[0]);
  }
};

template <typename T>
struct PcgDot {  // generic preconditioner: <r,z> after z = M^-1 r
  static constexpr int NDOT = 1;
  const T *r, *z; St<T> *st;
  __device__ bool skip() const { return st->done != kRunning; }
  __device__ NoScal load() const { return {}; }
  __device__ void apply(size_t i, NoScal, T (&d)[1]) const { d[0] += r[i] * z[i]; }
  __device__ void finalize(const T (&s)[1]) const { pcg_check(st, s[0]); }
};

template <typename T>
struct PcgP {  // p = z + beta p (z = r/d stored by PcgUpdate for Jacobi)
  static constexpr int NDOT = 0;
  T *p; const T *z; St<T> *st;
  struct S { T b; };
  __device__ bool skip() const { return st->done != kRunning; }
  __device__ S load() const { return {st->beta}; }
  __device__ void apply(size_t i, S s, T (&)[1]) const { p[i] = z[i] + s.b * p[i]; }
  __device__ void finalize(const T (&)[1]) const {}
};

// ===========================================================================
// pipelined BiCGStab (bicgstab.hpp:96-215, host_based/iterative_operations.hpp:519-627)
// ===========================================================================
template <typename T>
struct BicgInit {
  static constexpr int NDOT = 1;
  const T *b; T *x, *r, *p, *r0; St<T> *st;
  __device__ bool skip() const { return false; }
  __device__ NoScal load() const { return {}; }
  __device__ void apply(size_t i, NoScal, T (&d)[1]) const {
    T bi = b[i];
    x[i] = T(0); r[i] = bi; p[i] = bi; r0[i] = bi;
    d[0] += bi * bi;
  }
  __device__ void finalize(const T (&s)[1]) const {
    T nrm = sqrt(s[0]);
    st->nrhs = nrm;
    st->resnorm = nrm;
    st->r_r0 = nrm * nrm;
    st->iters = 0;
    st->error = 0;
    st->done = ((double)nrm <= st->abs_tol) ? kConverged : kRunning;
    if (st->done == kRunning && st->max_iters == 0) { st->done = kMaxIters; st->error = 1.0; }
  }
};

template <typename T>
struct EpiBicgAp {  // Ap = A p, <Ap, r0*>
  static constexpr int NDOT = 1;
  T *Ap; const T *r0; St<T> *st;
  struct Pre { T r0; };
  __device__ bool skip() const { return st->done != kRunning; }
  __device__ Pre pre(uint32_t r) const { return {r0[r]}; }
  __device__ void row(uint32_t r, T acc, const Pre &v, T (&d)[1]) const {
    Ap[r] = acc;
    d[0] += acc * v.r0;
  }
  __device__ void finalize(const T (&s)[1]) const {
    st->iters += 1;
    st->Ap_r0 = s[0];
    st->alpha = st->r_r0 / s[0];  // once here, not in every thread of BicgS
  }
};

template <typename T>
// s = r - alpha Ap (alpha = <r,r0*>/<Ap,r0*>); <s,s> comes from the next
// product's epilogue, which reads the same s (one grid reduction fewer)
struct BicgS {
  static constexpr int NDOT = 0;
  T *s_; const T *r, *Ap; St<T> *st;
  struct S { T a; };
  __device__ bool skip() const { return st->done != kRunning; }
  __device__ S load() const { return {st->alpha}; }
  __device__ void apply(size_t i, S s, T (&)[1]) const { s_[i] = r[i] - s.a * Ap[i]; }
  __device__ void finalize(const T (&)[1]) const {}
};

template <typename T>
struct EpiBicgAs {  // As = A s, <As,As>, <s,As>, <As,r0*>, <s,s>; scalars; residual estimate
  static constexpr int NDOT = 4;
  T *As; const T *s_, *r0; St<T> *st;
  struct Pre { T s, r0; };
  __device__ bool skip() const { return st->done != kRunning; }
  __device__ Pre pre(uint32_t r) const { return {s_[r], r0[r]}; }
  __device__ void row(uint32_t r, T acc, const Pre &v, T (&d)[4]) const {
    As[r] = acc;
    d[0] += acc * acc;
    d[1] += v.s * acc;
    d[2] += acc * v.r0;
    d[3] += v.s * v.s;
  }
  __device__ void finalize(const T (&s)[4]) const {
    st->s_s = s[3];
    T alpha = st->r_r0 / st->Ap_r0;
    T beta = -s[2] / st->Ap_r0;
    T omega = s[1] / s[0];
    T rn = sqrt(st->s_s - T(2) * omega * s[1] + omega * omega * s[0]);
    st->alpha = alpha;
    st->beta = beta;
    st->omega = omega;
    st->resnorm = rn;
    st->error = (double)rn / (double)st->nrhs;
    if (fabs((double)rn / (double)st->nrhs) < st->tol || (double)rn < st->abs_tol) {
      st->done = kConverged;  // leaves before the x update, as bicgstab.hpp:197-198
    } else if (!finite_(alpha) || !finite_(omega) || !finite_(beta)) {
      st->done = kBreakdown;
    }
  }
};

template <typename T>
struct BicgUpdate {  // x += a p + w s; r = s - w As; p = r + b (p - w Ap); <r, r0*>
  static constexpr int NDOT = 1;
  T *x, *p, *r; const T *s_, *As, *Ap, *r0; St<T> *st;
  struct S { T a, w, b; };
  __device__ bool skip() const { return st->done != kRunning; }
  __device__ S load() const { return {st->alpha, st->omega, st->beta}; }
  __device__ void apply(size_t i, S c, T (&d)[1]) const {
    T vp = p[i], vs = s_[i];
    x[i] += c.a * vp + c.w * vs;
    T vr = vs - c.w * As[i];
    vp = vr + c.b * (vp - c.w * Ap[i]);
    d[0] += vr * r0[i];
    r[i] = vr;
    p[i] = vp;
  }
  __device__ void finalize(const T (&s)[1]) const {
    st->r_r0 = s[0];
    if (st->iters >= st->max_iters) st->done = kMaxIters;
  }
};

// ===========================================================================
// preconditioned BiCGStab (bicgstab.hpp:398-489)
// ===========================================================================
template <typename T>
struct GbInit {  // x = 0; ||b||; restart at the first iteration
  static constexpr int NDOT = 1;
  const T *b; T *x; St<T> *st;
  __device__ bool skip() const { return false; }
  __device__ NoScal load() const { return {}; }
  __device__ void apply(size_t i, NoScal, T (&d)[1]) const {
    T bi = b[i];
    x[i] = T(0);
    d[0] += bi * bi;
  }
  __device__ void finalize(const T (&s)[1]) const {
    T nrm = sqrt(s[0]);
    st->nrhs = nrm;
    st->resnorm = nrm;
    st->iters = 0;
    st->error = 0;
    st->restart = 1;
    st->done = ((double)nrm <= st->abs_tol) ? kConverged : kRunning;
    if (st->done == kRunning && st->max_iters == 0) { st->done = kMaxIters; st->error = 1.0; }
    st->restart_skip = st->done != kRunning;
  }
};

template <typename T>
__device__ __forceinline__ void gb_restart_done(St<T> *st, T rr) {
  T nr = sqrt(rr);
  st->ip = nr * nr;
  st->restart = 0;
  st->restart_skip = 1;
  st->last_restart = st->iters;
}

template <typename T, bool JAC>
struct EpiGbRestart {  // r = M^-1 (b - A x) (Jacobi fused, else raw); p = r; r0* = r; ||r||^2
  static constexpr int NDOT = JAC ? 1 : 0;
  static constexpr bool jacobi = JAC;
  T *r, *p, *r0; const T *b, *dg; St<T> *st;
  struct Pre { T b, d; };
  __device__ bool skip() const { return st->restart_skip != 0; }
  __device__ Pre pre(uint32_t i) const { return {b[i], jacobi ? dg[i] : T(1)}; }
  __device__ void row(uint32_t i, T acc, const Pre &pv, T (&d)[1]) const {
    T v = pv.b - acc;
    if constexpr (JAC) {
      v = v * pv.d;
      p[i] = v;
      r0[i] = v;
      d[0] += v * v;
    }
    r[i] = v;
  }
  __device__ void finalize(const T (&s)[1]) const {
    if constexpr (JAC) gb_restart_done(st, s[0]);
  }
};

template <typename T>
struct GbRestartFinish {  // generic preconditioner: p = r0* = r (already M^-1 applied)
  static constexpr int NDOT = 1;
  T *p, *r0; const T *r; St<T> *st;
  __device__ bool skip() const { return st->restart_skip != 0; }
  __device__ NoScal load() const { return {}; }
  __device__ void apply(size_t i, NoScal, T (&d)[1]) const {
    T v = r[i];
    p[i] = v;
    r0[i] = v;
    d[0] += v * v;
  }
  __device__ void finalize(const T (&s)[1]) const { gb_restart_done(st, s[0]); }
};

template <typename T>
struct EpiStore {  // y = acc
  static constexpr int NDOT = 0;
  T *y; const int *flag;
  VCLGB_NO_PRE
  __device__ bool skip() const { return flag && *flag != kRunning; }
  __device__ void row(uint32_t i, T acc, const Pre &, T (&)[1]) const { y[i] = acc; }
  __device__ void finalize(const T (&)[1]) const {}
};

template <typename T>
struct EpiGb1 {  // t0 = M^-1 A p (Jacobi fused); <t0, r0*> -> alpha
  static constexpr int NDOT = 1;
  T *t0; const T *dg, *r0; St<T> *st;
  struct Pre { T d, r0; };
  __device__ bool skip() const { return st->done != kRunning; }
  __device__ Pre pre(uint32_t i) const { return {dg[i], r0[i]}; }
  __device__ void row(uint32_t i, T acc, const Pre &pv, T (&d)[1]) const {
    T v = acc * pv.d;
    t0[i] = v;
    d[0] += v * pv.r0;
  }
  __device__ void finalize(const T (&s)[1]) const {
    st->iters += 1;
    st->alpha = st->ip / s[0];
  }
};

template <typename T>
struct GbDot1 {  // generic: <t0, r0*> -> alpha
  static constexpr int NDOT = 1;
  const T *t0, *r0; St<T> *st;
  __device__ bool skip() const { return st->done != kRunning; }
  __device__ NoScal load() const { return {}; }
  __device__ void apply(size_t i, NoScal, T (&d)[1]) const { d[0] += t0[i] * r0[i]; }
  __device__ void finalize(const T (&s)[1]) const {
    st->iters += 1;
    st->alpha = st->ip / s[0];
  }
};

template <typename T>
struct GbS {  // s = r - alpha t0
  static constexpr int NDOT = 0;
  T *s_; const T *r, *t0; St<T> *st;
  struct S { T a; };
  __device__ bool skip() const { return st->done != kRunning; }
  __device__ S load() const { return {st->alpha}; }
  __device__ void apply(size_t i, S c, T (&)[1]) const { s_[i] = r[i] - c.a * t0[i]; }
  __device__ void finalize(const T (&)[1]) const {}
};

template <typename T>
__device__ __forceinline__ void gb_omega(St<T> *st, T t1t1, T t1s) {
  T nt1 = sqrt(t1t1);
  st->omega = t1s / (nt1 * nt1);
}

template <typename T>
struct EpiGb2 {  // t1 = M^-1 A s (Jacobi fused); ||t1||^2, <t1,s> -> omega
  static constexpr int NDOT = 2;
  T *t1; const T *dg, *s_; St<T> *st;
  struct Pre { T d, s; };
  __device__ bool skip() const { return st->done != kRunning; }
  __device__ Pre pre(uint32_t i) const { return {dg[i], s_[i]}; }
  __device__ void row(uint32_t i, T acc, const Pre &pv, T (&d)[2]) const {
    T v = acc * pv.d;
    t1[i] = v;
    d[0] += v * v;
    d[1] += v * pv.s;
  }
  __device__ void finalize(const T (&s)[2]) const { gb_omega(st, s[0], s[1]); }
};

template <typename T>
struct GbDot2 {
  static constexpr int NDOT = 2;
  const T *t1, *s_; St<T> *st;
  __device__ bool skip() const { return st->done != kRunning; }
  __device__ NoScal load() const { return {}; }
  __device__ void apply(size_t i, NoScal, T (&d)[2]) const {
    T v = t1[i];
    d[0] += v * v;
    d[1] += v * s_[i];
  }
  __device__ void finalize(const T (&s)[2]) const { gb_omega(st, s[0], s[1]); }
};

template <typename T>
struct GbUpdate {  // x += a p + w s; r = s - w t1; ||r||, <r,r0*>; beta, restart test
  static constexpr int NDOT = 2;
  T *x, *r; const T *p, *s_, *t1, *r0; St<T> *st;
  struct S { T a, w; };
  __device__ bool skip() const { return st->done != kRunning; }
  __device__ S load() const { return {st->alpha, st->omega}; }
  __device__ void apply(size_t i, S c, T (&d)[2]) const {
    T vs = s_[i];
    x[i] += c.a * p[i] + c.w * vs;
    T vr = vs - c.w * t1[i];
    r[i] = vr;
    d[0] += vr * vr;
    d[1] += vr * r0[i];
  }
  __device__ void finalize(const T (&s)[2]) const {
    T rn = sqrt(s[0]);
    st->resnorm = rn;
    st->error = (double)rn / (double)st->nrhs;
    if ((double)rn / (double)st->nrhs < st->tol || (double)rn < st->abs_tol) {
      st->done = kConverged;
      st->restart_skip = 1;
      return;
    }
    T new_ip = s[1];
    T beta = new_ip / st->ip * st->alpha / st->omega;
    st->beta = beta;
    st->ip = new_ip;
    unsigned i = st->iters - 1;
    if ((new_ip >= T(0) && new_ip <= T(0)) || (st->omega >= T(0) && st->omega <= T(0)) ||
        i - st->last_restart > st->max_before_restart) {
      st->restart = 1;
    }
    if (!finite_(st->alpha) || !finite_(st->omega)) st->done = kBreakdown;
    else if (st->iters >= st->max_iters) st->done = kMaxIters;
    st->restart_skip = (st->done != kRunning) || !st->restart;
  }
};

template <typename T>
struct GbP {  // p = r + beta (p - omega t0)
  static constexpr int NDOT = 0;
  T *p; const T *r, *t0; St<T> *st;
  struct S { T b, w; };
  __device__ bool skip() const { return st->done != kRunning; }
  __device__ S load() const { return {st->beta, st->omega}; }
  __device__ void apply(size_t i, S c, T (&)[1]) const {
    p[i] = r[i] + c.b * (p[i] - c.w * t0[i]);
  }
  __device__ void finalize(const T (&)[1]) const {}
};

// ===========================================================================
// pipelined GMRES (gmres.hpp:181-367, host_based/iterative_operations.hpp:734-935)
// ===========================================================================
constexpr int kGmresMaxK = 64;

template <typename T>
struct Gm {  // GMRES device state
  T nrhs, rho0, rho, vnorm2;
  T inv_rho0, inv_vnorm;  // 1/rho0, 1/||v_k||: formed once, the passes multiply
  T R[kGmresMaxK * kGmresMaxK];
  T xi[kGmresMaxK];
  T h[kGmresMaxK];
  T coef[kGmresMaxK];
  int kk;             // number of update coefficients
  unsigned restart_count, max_restarts;
  double tol, abs_tol, error;
  unsigned iters;
  unsigned K;
  int done;
};

template <typename T>
struct GmInit {
  static constexpr int NDOT = 1;
  const T *b; T *x, *r; Gm<T> *g;
  __device__ bool skip() const { return false; }
  __device__ NoScal load() const { return {}; }
  __device__ void apply(size_t i, NoScal, T (&d)[1]) const {
    T bi = b[i];
    x[i] = T(0);
    r[i] = bi;
    d[0] += bi * bi;
  }
  __device__ void finalize(const T (&s)[1]) const {
    g->nrhs = sqrt(s[0]);
    g->rho0 = g->nrhs;
    g->inv_rho0 = T(1) / g->rho0;
    g->rho = T(1);
    g->iters = 0;
    g->error = 0;
    g->restart_count = 0;
    g->done = kRunning;
  }
};

template <typename T>
__device__ __forceinline__ void gm_cycle_check(Gm<T> *g) {
  // gmres.hpp:226-233 (the restart bound ends the loop after the last cycle)
  if ((double)g->rho0 <= g->abs_tol) { g->done = kConverged; return; }
  g->rho = T(1);
  if ((double)(g->rho0 / g->nrhs) < g->tol || (double)g->rho0 < g->abs_tol) {
    g->done = kConverged;
    return;
  }
  if (g->restart_count > g->max_restarts) g->done = kMaxIters;
}

template <typename T>
struct GmCheckFirst {
  Gm<T> *g;
  __device__ void operator()() const { gm_cycle_check(g); }
};

template <typename T>
struct EpiGmResid {  // r = b - A x; rho0 = ||r||
  static constexpr int NDOT = 1;
  T *r; const T *b; Gm<T> *g;
  struct Pre { T b; };
  __device__ bool skip() const { return g->done != kRunning; }
  __device__ Pre pre(uint32_t i) const { return {b[i]}; }
  __device__ void row(uint32_t i, T acc, const Pre &pv, T (&d)[1]) const {
    T v = pv.b - acc;
    r[i] = v;
    d[0] += v * v;
  }
  __device__ void finalize(const T (&s)[1]) const {
    g->rho0 = sqrt(s[0]);
    g->inv_rho0 = T(1) / g->rho0;
    gm_cycle_check(g);
  }
};

template <typename T>
struct GmScaleR {  // r /= rho0 (the reference scales before its convergence test)
  static constexpr int NDOT = 0;
  T *r; Gm<T> *g;
  struct S { T inv; };
  __device__ bool skip() const { return false; }
  __device__ S load() const { return {g->inv_rho0}; }
  __device__ void apply(size_t i, S c, T (&)[1]) const { r[i] *= c.inv; }
  __device__ void finalize(const T (&)[1]) const {}
};

// v_k = A src for k > 0: the Gram-Schmidt pass reduces ||w||^2 after, so the
// product carries no reduction
template <typename T>
struct EpiGmVStore {
  static constexpr int NDOT = 0;
  T *vk; Gm<T> *g;
  VCLGB_NO_PRE
  __device__ bool skip() const { return g->done != kRunning; }
  __device__ void row(uint32_t i, T acc, const Pre &, T (&)[1]) const { vk[i] = acc; }
  __device__ void finalize(const T (&)[1]) const {}
};

template <typename T>
struct EpiGmV {  // v_0 = A r with ||v_0||^2 and <r, v_0> (k = 0): R(0,0), xi_0
  static constexpr int NDOT = 2;
  T *vk; const T *r; Gm<T> *g;
  VCLGB_NO_PRE
  __device__ bool skip() const { return g->done != kRunning; }
  __device__ void row(uint32_t i, T acc, const Pre &, T (&d)[2]) const {
    vk[i] = acc;
    d[0] += acc * acc;
    d[1] += r[i] * acc;
  }
  __device__ void finalize(const T (&s)[2]) const {
    const T inv = T(1) / sqrt(s[0]);
    g->vnorm2 = s[0];
    g->inv_vnorm = inv;
    g->R[0] = sqrt(s[0]);
    g->xi[0] = s[1] * inv;
  }
};

// ---------------------------------------------------------------------------
// Classical Gram-Schmidt over the first k columns of a basis Q (leading
// dimension ld), shared by both GMRES forms: the multi-dot h_j = <Q_j, w>,
// j < k (one pass over the basis, a tall-skinny GEMV) and the update
// w -= sum_j h_j Q_j with ||w||^2.  On GB300 these passes are bound by the
// FP64 pipe (2 FMAs per clock per SM; k FMAs per row against (k+1)*8 bytes),
// so only the FMAs the algorithm needs are issued: the column loops are
// unrolled to the exact count (a guard j < k inside a loop unrolled to a
// larger bound still issued the guarded FMAs -- measured 77 us against 31 us
// at k = 2 on 4M rows), and each row's column loads are issued before its
// FMAs.  The multi-dot runs one group of up to kCgsCols columns per
// blockIdx.y; the update walks the columns in chunks of kCgsCols, subtracting
// in column order as a single loop would.
// ---------------------------------------------------------------------------
constexpr int kCgsCols = 8;

template <typename T, int C>
__device__ __forceinline__ void cgs_dot_rows(size_t n, const T *__restrict__ Q, size_t ld,
                                             const T *__restrict__ w, T *red) {
  T acc[C];
#pragma unroll
  for (int j = 0; j < C; ++j) acc[j] = T(0);
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const T v = w[i];
    T q[C];
#pragma unroll
    for (int j = 0; j < C; ++j) q[j] = Q[(size_t)j * ld + i];
#pragma unroll
    for (int j = 0; j < C; ++j) acc[j] += q[j] * v;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < C; ++j) {
    const T t = warp_sum(acc[j]);
    if (lane == 0) red[j * 8 + warp] = t;
  }
}

// Out: skip(), store(j, h_j).  Grid (blocks per group, column groups), 256
// threads; partials[j * gridDim.x + block] holds each block's share of h_j.
template <typename T, class Out>
__global__ void __launch_bounds__(256)
    cgs_multidot_kernel(size_t n, int k, const T *__restrict__ Q, size_t ld,
                        const T *__restrict__ w, Out out, T *partials, unsigned *counter) {
  if (out.skip()) return;
  __shared__ T red[kCgsCols * 8];
  __shared__ bool am_last;
  const int j0 = kCgsCols * (int)blockIdx.y;
  const int c = min(kCgsCols, k - j0);
  const T *Qg = Q + (size_t)j0 * ld;
  switch (c) {
    case 1: cgs_dot_rows<T, 1>(n, Qg, ld, w, red); break;
    case 2: cgs_dot_rows<T, 2>(n, Qg, ld, w, red); break;
    case 3: cgs_dot_rows<T, 3>(n, Qg, ld, w, red); break;
    case 4: cgs_dot_rows<T, 4>(n, Qg, ld, w, red); break;
    case 5: cgs_dot_rows<T, 5>(n, Qg, ld, w, red); break;
    case 6: cgs_dot_rows<T, 6>(n, Qg, ld, w, red); break;
    case 7: cgs_dot_rows<T, 7>(n, Qg, ld, w, red); break;
    default: cgs_dot_rows<T, 8>(n, Qg, ld, w, red); break;
  }
  __syncthreads();
  const unsigned nb = gridDim.x;
  for (int j = threadIdx.x; j < c; j += blockDim.x) {
    T t = 0;
    for (int q = 0; q < 8; ++q) t += red[j * 8 + q];
    partials[(size_t)(j0 + j) * nb + blockIdx.x] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // one acquire-release ticket (the barrier above orders the block's
    // partial writes before it, the one below the last block's reads after)
    cuda::atomic_ref<unsigned, cuda::thread_scope_device> ticket(*counter);
    am_last = ticket.fetch_add(1u, cuda::memory_order_acq_rel) == gridDim.x * gridDim.y - 1;
  }
  __syncthreads();
  if (!am_last) return;
  // last block: one warp per projection, partials read at L2 in a fixed order
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int j = warp; j < k; j += 8) {
    T t = 0;
    for (unsigned b = lane; b < nb; b += 32) t += __ldcg(partials + (size_t)j * nb + b);
    t = warp_sum(t);
    if (lane == 0) out.store(j, t);
  }
  if (threadIdx.x == 0) *counter = 0;
}

template <typename T, int C>
__device__ __forceinline__ T cgs_sub_cols(T v, const T *__restrict__ Q, size_t ld, size_t i,
                                          const T *hs) {
  T q[C];
#pragma unroll
  for (int j = 0; j < C; ++j) q[j] = Q[(size_t)j * ld + i];
#pragma unroll
  for (int j = 0; j < C; ++j) v -= hs[j] * q[j];
  return v;
}

// d[0] += ||w||^2 and, for ND == 2, d[1] += <r, w> (w after the update)
template <typename T, int TAIL, int ND>
__device__ __forceinline__ void cgs_orth_rows(size_t n, int full, const T *__restrict__ Q,
                                              size_t ld, T *__restrict__ w, const T *hs,
                                              const T *__restrict__ r, T (&d)[ND]) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    T v = w[i];
    for (int c = 0; c < full; ++c)
      v = cgs_sub_cols<T, kCgsCols>(v, Q + (size_t)c * kCgsCols * ld, ld, i, hs + c * kCgsCols);
    if constexpr (TAIL > 0)
      v = cgs_sub_cols<T, TAIL>(v, Q + (size_t)full * kCgsCols * ld, ld, i, hs + full * kCgsCols);
    d[0] += v * v;
    if constexpr (ND == 2) d[1] += r[i] * v;
    w[i] = v;
  }
}

// Fin: NDOT (1: ||w||^2; 2: also <r, w> with r = dot_with()), skip(), h(j)
// (the projections), finalize(sums)
template <typename T, class Fin>
__global__ void __launch_bounds__(256)
    cgs_orth_kernel(size_t n, int k, const T *__restrict__ Q, size_t ld, T *__restrict__ w, Fin fin,
                    T *partials, unsigned *counter) {
  constexpr int ND = Fin::NDOT;
  if (fin.skip()) return;
  __shared__ T hs[kGmresMaxK];
  __shared__ T smem[ND * 256];  // block_sum_wide over 256 threads
  for (int j = threadIdx.x; j < k; j += blockDim.x) hs[j] = fin.h(j);
  __syncthreads();
  const int full = k / kCgsCols;
  const T *r = fin.dot_with();
  T d[ND];
#pragma unroll
  for (int i = 0; i < ND; ++i) d[i] = T(0);
  switch (k % kCgsCols) {
    case 0: cgs_orth_rows<T, 0, ND>(n, full, Q, ld, w, hs, r, d); break;
    case 1: cgs_orth_rows<T, 1, ND>(n, full, Q, ld, w, hs, r, d); break;
    case 2: cgs_orth_rows<T, 2, ND>(n, full, Q, ld, w, hs, r, d); break;
    case 3: cgs_orth_rows<T, 3, ND>(n, full, Q, ld, w, hs, r, d); break;
    case 4: cgs_orth_rows<T, 4, ND>(n, full, Q, ld, w, hs, r, d); break;
    case 5: cgs_orth_rows<T, 5, ND>(n, full, Q, ld, w, hs, r, d); break;
    case 6: cgs_orth_rows<T, 6, ND>(n, full, Q, ld, w, hs, r, d); break;
    default: cgs_orth_rows<T, 7, ND>(n, full, Q, ld, w, hs, r, d); break;
  }
  T s[ND];
  if (grid_reduce<ND, true>(d, partials, counter, smem, s)) fin.finalize(s);
}

// One Gram-Schmidt pass (multi-dot, then update) of w against Q's first k
// columns; both grids are capped at one wave of their kernel.
template <typename T, class Out, class Fin>
static void cgs_pass(Backend &be, size_t n, int k, const T *Q, size_t ld, T *w, const Out &out,
                     const Fin &fin, T *partials, unsigned *counter) {
  const int groups = (k + kCgsCols - 1) / kCgsCols;
  const int want = vec_grid(be, n);
  const int md_wave = one_wave<cgs_multidot_kernel<T, Out>>(be, 1 << 30, 256);
  const int gx = std::max(1, std::min(want, md_wave / groups));
  cgs_multidot_kernel<T, Out><<<dim3(gx, groups), 256, 0, be.stream>>>(n, k, Q, ld, w, out,
                                                                       partials, counter);
  const int go = one_wave<cgs_orth_kernel<T, Fin>>(be, want, 256);
  cgs_orth_kernel<T, Fin><<<go, 256, 0, be.stream>>>(n, k, Q, ld, w, fin, partials, counter);
  be.launches += 2;
  VCLGB_CHECK_LAUNCH();
}

// unpreconditioned GMRES: h_j = <v_j, v_k> into h and R(:,k); ||v_k||^2
template <typename T>
struct GmDots {
  Gm<T> *g; int k;
  __device__ bool skip() const { return g->done != kRunning; }
  __device__ void store(int j, T t) const {
    g->h[j] = t;
    g->R[j + (size_t)k * g->K] = t;
  }
};
// ||w||^2 and <r, w> of the orthogonalised w give R(k,k) = ||w|| and
// xi_k = <r, w> / ||w|| = <r, v_k> without a reduction over the normalised v_k
template <typename T>
struct GmOrthEnd {
  static constexpr int NDOT = 2;
  Gm<T> *g; const T *r; int k;
  __device__ bool skip() const { return g->done != kRunning; }
  __device__ T h(int j) const { return g->h[j]; }
  __device__ const T *dot_with() const { return r; }
  __device__ void finalize(const T (&s)[2]) const {
    const T inv = T(1) / sqrt(s[0]);
    g->vnorm2 = s[0];
    g->inv_vnorm = inv;
    g->R[k + (size_t)k * g->K] = sqrt(s[0]);
    g->xi[k] = s[1] * inv;
  }
};

template <typename T>
struct GmNormalize {  // v_k /= ||v_k|| (R(k,k) and xi_k came with ||v_k||)
  static constexpr int NDOT = 0;
  T *vk; Gm<T> *g;
  struct S { T nv; };
  __device__ bool skip() const { return g->done != kRunning; }
  __device__ S load() const { return {g->inv_vnorm}; }
  __device__ void apply(size_t i, S c, T (&)[1]) const {
    vk[i] *= c.nv;  // times 1/||v_k||, formed once by the kernel before
  }
  __device__ void finalize(const T (&)[1]) const {}
};

// the host part of a restart cycle (gmres.hpp:287-345) as one device thread
template <typename T>
struct GmCycleEnd {
  Gm<T> *g;
  __device__ void operator()() const {
    if (g->done != kRunning) { g->kk = 0; return; }
    const unsigned K = g->K;
    unsigned k = K, full_k = K;
    for (unsigned i = 0; i < k; ++i)
      if (fabs((double)g->R[i + i * k]) < g->tol * (double)g->R[0]) { k = i; break; }
    T rho = g->rho;
    for (unsigned i = 0; i < k; ++i) {
      g->iters += 1;
      T xi = g->xi[i];
      if (xi >= rho || xi <= -rho) { k = i; break; }
      rho *= sin(acos(xi / rho));
    }
    g->rho = rho;
    T eta[kGmresMaxK];
    for (unsigned i = 0; i < K; ++i) eta[i] = g->xi[i];
    for (int i2 = (int)k - 1; i2 > -1; --i2) {
      unsigned i = (unsigned)i2;
      for (unsigned j = i + 1; j < k; ++j) eta[i] -= g->R[i + j * full_k] * eta[j];
      eta[i] /= g->R[i + i * full_k];
    }
    for (unsigned i = 0; i < k; ++i) g->coef[i] = g->rho0 * eta[i];
    g->kk = (int)k;
    g->error = fabs((double)(rho * g->rho0 / g->nrhs));
    g->restart_count += 1;
  }
};

template <typename T>
struct GmUpdateX {  // x += c0 r + sum_{j>=1} c_j v_{j-1}
  static constexpr int NDOT = 0;
  T *x; const T *r, *V; size_t ld; Gm<T> *g;
  struct S { int kk; };
  __device__ bool skip() const { return g->done != kRunning || g->kk == 0; }
  __device__ S load() const { return {g->kk}; }
  __device__ void apply(size_t i, S c, T (&)[1]) const {
    T v = x[i] + g->coef[0] * r[i];
    for (int j = 1; j < c.kk; ++j) v += g->coef[j] * V[(size_t)(j - 1) * ld + i];
    x[i] = v;
  }
  __device__ void finalize(const T (&)[1]) const {}
};

// ===========================================================================
// preconditioned GMRES: the control flow of the reference's Householder
// "simpler GMRES" (gmres.hpp:449-631, Walker): r = M^-1 (b - A x) and the
// stopping test at every restart, an iteration count per Krylov step, the
// clamped projection xi_k and the test |rho rho_0 / ||b||| < tol after every
// step, the triangular solve and x += rho_0 (eta_0 r + sum eta_j q_{j-1}).
// The orthonormal basis is the same one the reflections build (in exact
// arithmetic the k-th column of P_0 ... P_k is q_k and R(:,k) = Q^T w,
// ||w - Q Q^T w||); it is formed by classical Gram-Schmidt in one pass over
// the basis (a tall-skinny GEMV) and repeated once when the first pass
// cancelled more than half of ||w||^2 (the DGKS test, "twice is enough"),
// which keeps the basis as orthogonal as the reflections do.  Every step
// costs a few grid-wide passes instead of 2k reflections (an inner product
// and an axpy each, one after the other).
// ===========================================================================
template <typename T>
struct Gh {  // device state of the preconditioned GMRES
  T nrhs, rho0, inv_rho0, rho, wnorm2, vnorm2, inv_vnorm;
  T R[kGmresMaxK * kGmresMaxK];  // column k at R[k * K ...]: Q^T w, then ||w'|| at row k
  T proj[kGmresMaxK];
  T h[kGmresMaxK];
  T coef[kGmresMaxK];
  int kk;                        // steps taken in the current cycle
  int lost;                      // the cycle ended at the clamp of xi (see gh_step)
  int upd;                       // coefficients pending for the x update
  int pending;                   // status to take after the update (0: keep running)
  unsigned restart_count, max_restarts;
  double tol, abs_tol, error;
  unsigned iters, K;
  int done;
  int step_skip;                 // done || the cycle stopped
  int reorth_skip;               // step_skip || no second Gram-Schmidt pass needed
  int step_at;                   // the step whose stopping test ran last (-1: none)
};

template <typename T>
struct GhInit {  // x = 0; ||b||
  static constexpr int NDOT = 1;
  const T *b; T *x; Gh<T> *g;
  __device__ bool skip() const { return false; }
  __device__ NoScal load() const { return {}; }
  __device__ void apply(size_t i, NoScal, T (&d)[1]) const {
    const T bi = b[i];
    x[i] = T(0);
    d[0] += bi * bi;
  }
  __device__ void finalize(const T (&s)[1]) const {
    g->nrhs = sqrt(s[0]);
    g->iters = 0;
    g->error = 0;
    g->restart_count = 0;
    g->upd = 0;
    g->pending = 0;
    g->done = ((double)g->nrhs <= g->abs_tol) ? kConverged : kRunning;
    g->step_skip = 1;
    g->reorth_skip = 1;
    g->step_at = -1;
  }
};

// cycle start (gmres.hpp:484-510): rho_0 = ||M^-1 (b - A x)||, premature
// convergence test, then rho = 1 and a fresh cycle
template <typename T>
__device__ __forceinline__ void gh_cycle_start(Gh<T> *g, T rr) {
  const T rho0 = sqrt(rr);
  g->step_at = -1;
  g->rho0 = rho0;
  if ((double)(rho0 / g->nrhs) < g->tol || (double)rho0 < g->abs_tol) {
    g->error = (double)(rho0 / g->nrhs);
    g->done = kConverged;
    g->step_skip = 1;
    g->reorth_skip = 1;
    return;
  }
  g->inv_rho0 = T(1) / rho0;
  g->rho = T(1);
  g->kk = 0;
  g->lost = 0;
  g->step_skip = 0;
  g->reorth_skip = 1;
  if (!finite_(rho0)) { g->done = kBreakdown; g->step_skip = 1; }
}

// A step's stopping test (gmres.hpp:570-590), run by the reduction that gives
// the step's final ||w||^2 together with <r, w>: R(k,k) = ||w||, xi_k =
// <r, w> / ||w|| = <r, q_k>, the clamp of xi and the tolerance test.  step_at
// records the step, so that its normalisation still writes q_k when the test
// ends the cycle there.
template <typename T>
__device__ __forceinline__ void gh_step(Gh<T> *g, int k, T ww, T rw) {
  const T nv = sqrt(ww);
  if (!(nv > T(0)) || !finite_(nv)) {
    // w lies in the span of the basis (or is not finite): the cycle ends
    // with the k steps before this one
    g->step_skip = 1;
    g->reorth_skip = 1;
    if (!finite_(nv)) g->pending = kBreakdown;
    return;
  }
  g->step_at = k;
  g->R[(size_t)k * g->K + k] = nv;
  T xi = rw * g->inv_vnorm;
  const T rho = g->rho;
  // |xi| <= rho holds in exact arithmetic; the reference clamps xi to +-rho
  // ("machine precision reached", gmres.hpp:575-578), which makes rho 0 and
  // stops the solve as converged.  The estimate rho = sqrt(1 - sum xi^2) of
  // a residual normalised by its computed norm cannot resolve rho much below
  // sqrt(n eps), so the clamp can fire while the true residual is far above
  // the tolerance (seen: Jacobi GMRES on a 4M-row matrix whose M^-1 b is 467
  // times ||b||, true residual 3.6e-3 at "convergence").  Here the cycle ends
  // at the clamp without declaring convergence, and the next cycle's
  // residual r = M^-1 (b - A x), computed from x, decides.
  const bool clamped = xi >= rho || xi <= -rho;
  if (xi > rho) xi = rho;
  if (xi < -rho) xi = -rho;
  g->proj[k] = xi;
  const T nr = rho * sin(acos(xi / rho));
  g->rho = nr;
  g->kk = k + 1;
  if (clamped) {
    g->lost = 1;
    g->step_skip = 1;
    g->reorth_skip = 1;
  } else if (fabs((double)(nr * g->rho0 / g->nrhs)) < g->tol) {  // gmres.hpp:583-588
    g->step_skip = 1;
    g->reorth_skip = 1;
  }
}

template <typename T, bool JAC>
struct EpiGhResid {  // r = M^-1 (b - A x): Jacobi fused with ||r||^2, else raw b - A x
  static constexpr int NDOT = JAC ? 1 : 0;
  static constexpr bool jacobi = JAC;
  T *r; const T *b, *inv_d; Gh<T> *g;
  struct Pre { T b, id; };
  __device__ bool skip() const { return g->done != kRunning; }
  __device__ Pre pre(uint32_t i) const { return {b[i], jacobi ? inv_d[i] : T(1)}; }
  __device__ void row(uint32_t i, T acc, const Pre &pv, T (&d)[1]) const {
    T v = pv.b - acc;
    if constexpr (JAC) {
      v = v * pv.id;
      d[0] += v * v;
    }
    r[i] = v;
  }
  __device__ void finalize(const T (&s)[1]) const {
    if constexpr (JAC) gh_cycle_start(g, s[0]);
  }
};

template <typename T>
struct GhResidNorm {  // generic preconditioner: ||r||^2 after r = M^-1 r
  static constexpr int NDOT = 1;
  const T *r; Gh<T> *g;
  __device__ bool skip() const { return g->done != kRunning; }
  __device__ NoScal load() const { return {}; }
  __device__ void apply(size_t i, NoScal, T (&d)[1]) const { const T v = r[i]; d[0] += v * v; }
  __device__ void finalize(const T (&s)[1]) const { gh_cycle_start(g, s[0]); }
};

template <typename T>
struct GhScaleR {  // r /= rho_0
  static constexpr int NDOT = 0;
  T *r; Gh<T> *g;
  struct S { T inv; };
  __device__ bool skip() const { return g->step_skip != 0; }
  __device__ S load() const { return {g->inv_rho0}; }
  __device__ void apply(size_t i, S c, T (&)[1]) const { r[i] *= c.inv; }
  __device__ void finalize(const T (&)[1]) const {}
};

template <typename T>
__device__ __forceinline__ void gh_w_done(Gh<T> *g, T ww) {
  g->iters += 1;  // one Krylov step (gmres.hpp:522)
  g->wnorm2 = ww;
  g->vnorm2 = ww;
  g->inv_vnorm = T(1) / sqrt(ww);
}

// w = M^-1 A q with Jacobi fused: ||w||^2 and, at step 0 (RDOT, no
// Gram-Schmidt pass follows), <r, w> and the step's test; else the raw A q
template <typename T, bool JAC, bool RDOT>
struct EpiGhW {
  static constexpr int NDOT = JAC ? (RDOT ? 2 : 1) : 0;
  static constexpr bool jacobi = JAC;
  T *w; const T *inv_d, *r; Gh<T> *g;
  struct Pre { T id, r; };
  __device__ bool skip() const { return g->step_skip != 0; }
  __device__ Pre pre(uint32_t i) const {
    return {jacobi ? inv_d[i] : T(1), (JAC && RDOT) ? r[i] : T(0)};
  }
  __device__ void row(uint32_t i, T acc, const Pre &pv, T (&d)[DotArr<NDOT>::n]) const {
    if constexpr (JAC) {
      acc = acc * pv.id;
      d[0] += acc * acc;
      if constexpr (RDOT) d[1] += pv.r * acc;
    }
    w[i] = acc;
  }
  __device__ void finalize(const T (&s)[DotArr<NDOT>::n]) const {
    if constexpr (JAC) {
      gh_w_done(g, s[0]);
      if constexpr (RDOT) gh_step(g, 0, s[0], s[1]);
    }
  }
};

template <typename T, bool RDOT>
struct GhWNorm {  // generic preconditioner: ||w||^2 (and at step 0 <r, w>) after w = M^-1 A q
  static constexpr int NDOT = RDOT ? 2 : 1;
  const T *w, *r; Gh<T> *g;
  __device__ bool skip() const { return g->step_skip != 0; }
  __device__ NoScal load() const { return {}; }
  __device__ void apply(size_t i, NoScal, T (&d)[NDOT]) const {
    const T v = w[i];
    d[0] += v * v;
    if constexpr (RDOT) d[1] += r[i] * v;
  }
  __device__ void finalize(const T (&s)[NDOT]) const {
    gh_w_done(g, s[0]);
    if constexpr (RDOT) gh_step(g, 0, s[0], s[1]);
  }
};

// Gram-Schmidt for the preconditioned form.  SECOND: the re-orthogonalisation
// pass (skipped unless the DGKS test asked for it); its projections are added
// to R(:,k).  The first pass's update compares ||w'||^2 with ||w||^2 and
// requests the second pass when more than half of it cancelled.
template <typename T, bool SECOND>
struct GhDots {
  Gh<T> *g; int k;
  __device__ bool skip() const { return SECOND ? g->reorth_skip : g->step_skip; }
  __device__ void store(int j, T t) const {
    g->h[j] = t;
    if (SECOND) g->R[(size_t)k * g->K + j] += t;
    else g->R[(size_t)k * g->K + j] = t;
  }
};
// the pass that leaves no second pass to run ends the step: its reduction
// carries <r, w> for the step's test
template <typename T, bool SECOND>
struct GhOrthEnd {
  static constexpr int NDOT = 2;
  Gh<T> *g; const T *r; int k;
  __device__ bool skip() const { return SECOND ? g->reorth_skip : g->step_skip; }
  __device__ T h(int j) const { return g->h[j]; }
  __device__ const T *dot_with() const { return r; }
  __device__ void finalize(const T (&s)[2]) const {
    g->vnorm2 = s[0];
    g->inv_vnorm = T(1) / sqrt(s[0]);
    if (!SECOND) g->reorth_skip = !(s[0] < T(0.5) * g->wnorm2);
    else g->reorth_skip = 1;
    if (g->reorth_skip) gh_step(g, k, s[0], s[1]);
  }
};

// q_k = w / ||w||.  Skipped when the cycle stopped before this step; the step
// whose test stopped it (step_at) still writes its q_k, which the update uses.
template <typename T>
struct GhNormalize {
  static constexpr int NDOT = 0;
  T *q; const T *w; Gh<T> *g; int k;
  struct S { T inv; };
  __device__ bool skip() const { return g->step_skip != 0 && g->step_at != k; }
  __device__ S load() const { return {g->inv_vnorm}; }
  __device__ void apply(size_t i, S c, T (&)[1]) const { q[i] = w[i] * c.inv; }
  __device__ void finalize(const T (&)[1]) const {}
};

// end of a cycle (gmres.hpp:593-625) as one device thread: triangular solve,
// update coefficients, error, restart bookkeeping
template <typename T>
struct GhCycleEnd {
  Gh<T> *g;
  __device__ void operator()() const {
    if (g->done != kRunning) { g->upd = 0; return; }
    const unsigned K = g->K;
    const int k = g->kk;
    T eta[kGmresMaxK];
    for (int i = 0; i < k; ++i) eta[i] = g->proj[i];
    for (int i = k - 1; i > -1; --i) {
      for (int j = i + 1; j < k; ++j) eta[i] -= g->R[(size_t)j * K + i] * eta[j];
      eta[i] /= g->R[(size_t)i * K + i];
    }
    for (int i = 0; i < k; ++i) g->coef[i] = g->rho0 * eta[i];
    g->upd = k;
    g->error = fabs((double)(g->rho * g->rho0 / g->nrhs));
    g->restart_count += 1;
    if (g->pending == 0) {
      if (g->error < g->tol && !g->lost) g->pending = kConverged;
      else if (g->restart_count > g->max_restarts) g->pending = kMaxIters;
    }
    for (int i = 0; i < k; ++i)
      if (!finite_(g->coef[i])) { g->pending = kBreakdown; g->upd = 0; }
  }
};

template <typename T>
struct GhUpdateX {  // x += c0 r + sum_{j>=1} c_j q_{j-1}
  static constexpr int NDOT = 0;
  T *x; const T *r, *Q; size_t ld; Gh<T> *g;
  struct S { int kk; };
  __device__ bool skip() const { return g->done != kRunning || g->upd == 0; }
  __device__ S load() const { return {g->upd}; }
  __device__ void apply(size_t i, S c, T (&)[1]) const {
    T v = g->coef[0] * r[i];
    for (int j = 1; j < c.kk; ++j) v += g->coef[j] * Q[(size_t)(j - 1) * ld + i];
    x[i] += v;
  }
  __device__ void finalize(const T (&)[1]) const {}
};

template <typename T>
struct GhCycleClose {  // after the update: take the pending status
  Gh<T> *g;
  __device__ void operator()() const {
    g->upd = 0;
    g->step_at = -1;
    if (g->done == kRunning && g->pending != 0) {
      g->done = g->pending;
      g->step_skip = 1;
      g->reorth_skip = 1;
    }
  }
};

// ===========================================================================
// host drivers
// ===========================================================================
struct Workspace {
  DevBuf buf;
  std::vector<size_t> offs;
  size_t total = 0;
  size_t add(size_t bytes) {
    size_t o = total;
    total += (bytes + 255) / 256 * 256;
    offs.push_back(o);
    return o;
  }
  void commit(Backend &be) {
    buf.alloc(std::max<size_t>(total, 256), be.stream);
    VCLGB_CUDA(cudaMemsetAsync(buf.ptr, 0, buf.bytes, be.stream));
  }
  template <typename X> X *at(size_t off) const { return reinterpret_cast<X *>(buf.as<char>() + off); }
};

static inline uint32_t auto_check_every(const vclgbSolverTag *tag, uint32_t rows) {
  if (tag->check_every) return tag->check_every;
  if (rows < (1u << 16)) return 32;
  if (rows < (1u << 20)) return 16;
  return 8;
}

template <typename T>
static void set_tag_outputs(Backend &be, const St<T> *d_st, vclgbSolverTag *tag) {
  St<T> h;
  VCLGB_CUDA(cudaMemcpyAsync(&h, d_st, sizeof(h), cudaMemcpyDeviceToHost, be.stream));
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  tag->iters = h.iters;
  tag->error = h.error;
  tag->status = h.done == kConverged ? VCLGB_SUCCESS
              : h.done == kMaxIters  ? VCLGB_NOT_CONVERGED
                                     : VCLGB_BREAKDOWN;
}

template <typename T>
static St<T> make_state(const vclgbSolverTag *tag) {
  St<T> s;
  std::memset(&s, 0, sizeof(s));
  s.tol = tag->tol;
  s.abs_tol = tag->abs_tol;
  s.max_iters = tag->max_iters;
  s.max_before_restart = tag->max_iters_before_restart;
  return s;
}

static inline bool diag_needed(const Precond *P) { return P && P->kind == 1; }

// ===========================================================================
// Small systems in one thread-block cluster.  Below a few tens of thousands of
// rows a solver iteration is a chain of short kernels whose launch gaps and
// last-block reduction tails cost ~6 us each; here one cluster of up to 16
// CTAs runs every iteration.  Each CTA owns a contiguous chunk of rows (a row
// stays with one thread in every phase); a reduction is a block sum into a
// double-buffered shared slot, one cluster barrier (release/acquire), and a
// read of every CTA's slot through distributed shared memory in rank order,
// after which every CTA holds the same sums and runs the same scalar step
// (the expressions of CgInit/EpiCgFirst/CgUpdate/EpiCg and of the Jacobi PCG
// functors above, in the same types).  Values another CTA wrote (the search
// direction the products gather) are read at L2.  Nothing waits but the
// hardware cluster barrier; the loop ends at the solver's own iteration bound.
// ===========================================================================
constexpr uint32_t kClusterSolveThreads = 512;
// At most 2,048 rows a CTA (32,768 rows in a 16-CTA cluster): measured per
// iteration on the 2D Laplacian, CG takes 13.1 us at 2,048 rows a CTA and 19.5
// us at 4,096 (the per-phase path 16.1 us); BiCGStab 26.4 us against 32-37 us.
constexpr uint32_t kClusterSolveMaxRows = 32768;
constexpr uint32_t kClusterSolveMaxChunk = 2048;
constexpr size_t kClusterSolveSmem = 192 * 1024;  // dynamic shared memory a CTA, at most

// the scalar state of a cluster solve, kept by thread 0 of every CTA (each
// runs the same steps on the same sums) and read by the block after a barrier
template <typename T>
struct ClState {
  T part[2][16][4];  // every CTA's partial sums (by rank), double buffered by phase
  T warp[4 * 16];    // block_sum scratch (up to 4 values x 16 warps)
  T rr, nrhs2, alpha, beta, ip;
  T omega, nrhs, Ap_r0, s_s, r_r0;  // BiCGStab
  double error;
  unsigned iters, last_restart;
  int done;
  int restart;
  int buf;
};

__device__ __forceinline__ void cl_barrier() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
  asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

// The cluster sum of NV values per thread, then step(sums) on thread 0 of
// each CTA (it updates the shared state); the block sees the new state on
// return.  Each CTA pushes its block sums into every CTA's slot for its rank
// (distributed shared memory stores) before the barrier, so after it the
// sums are read locally, in rank order.  The scalar step runs once per CTA:
// FP64 divisions and square roots in every thread would cost more than the
// rows of a small system.
template <int NV, typename T, class F>
__device__ __forceinline__ void cl_step(T (&v)[NV], ClState<T> &cs, F &&step) {
  block_sum<NV>(v, cs.warp);
  const int b = cs.buf;
  cg::cluster_group cl = cg::this_cluster();
  const unsigned nct = cl.num_blocks(), me = cl.block_rank();
  if (threadIdx.x < 32) {
    T mine[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) mine[i] = __shfl_sync(0xffffffffu, v[i], 0);
    if (threadIdx.x < nct) {
      T *dst = cl.map_shared_rank(&cs.part[b][me][0], threadIdx.x);
#pragma unroll
      for (int i = 0; i < NV; ++i) dst[i] = mine[i];
    }
  }
  cl_barrier();
  if (threadIdx.x < 32) {
    const unsigned lane = threadIdx.x;
    T t[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) t[i] = lane < nct ? cs.part[b][lane][i] : T(0);
#pragma unroll
    for (int i = 0; i < NV; ++i) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) t[i] += __shfl_xor_sync(0xffffffffu, t[i], o);
    }
    if (lane == 0) {
      cs.buf = b ^ 1;
      step(t);
    }
  }
  __syncthreads();
}

// The vectors live in shared memory: CTA k holds rows [k << shift, (k+1) <<
// shift) of x, r, p, q (and z and the reciprocal diagonal for PCG); a
// product gathers p through distributed shared memory from the CTA that owns
// the column.  The loop touches no global memory but the matrix, so the
// cluster barrier's release orders only shared-memory writes.
template <typename T>
__device__ __forceinline__ T cl_row(const CsrView<T> &A, uint32_t i, const T *sp, uint32_t rank,
                                    uint32_t shift) {
  cg::cluster_group cl = cg::this_cluster();
  const uint32_t mask = (1u << shift) - 1;
  T acc = T(0);
  const uint32_t e = __ldg(A.rp + i + 1);
  for (uint32_t k = __ldg(A.rp + i); k < e; ++k) {
    const uint32_t c = __ldg(A.ci + k), owner = c >> shift;
    const T pc = owner == rank ? sp[c & mask] : *cl.map_shared_rank(sp + (c & mask), owner);
    acc += __ldg(A.v + k) * pc;
  }
  return acc;
}

// JAC false: pipelined CG (no preconditioner); true: PCG with the reciprocal
// diagonal dg (Jacobi, row scaling)
template <typename T, bool JAC>
__global__ void __launch_bounds__(kClusterSolveThreads, 1)
    cluster_cg_kernel(CsrView<T> A, const T *b, T *x, const T *dg, St<T> *st, uint32_t shift) {
  __shared__ ClState<T> cs;
  extern __shared__ __align__(16) unsigned char cl_vec_bytes[];
  cg::cluster_group cl = cg::this_cluster();
  const uint32_t rank = cl.block_rank(), len = 1u << shift;
  T *sx = reinterpret_cast<T *>(cl_vec_bytes), *sr = sx + len, *sp = sr + len, *sq = sp + len;
  T *sz = sq + len, *sd = sz + len;  // PCG only
  const uint32_t n = A.rows;
  const uint32_t r0 = min(rank << shift, n), r1 = min(r0 + len, n), m = r1 - r0;
  const double tol = st->tol, abs_tol = st->abs_tol;
  const unsigned max_iters = st->max_iters;
  if (threadIdx.x == 0) {
    cs.buf = 0;
    cs.iters = 0;
    cs.error = 0;
    cs.alpha = cs.beta = cs.rr = cs.ip = cs.nrhs2 = T(0);
  }
  if (!JAC) {
    T d[1] = {T(0)};
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
      const T bi = b[r0 + i];
      sx[i] = T(0); sr[i] = bi; sp[i] = bi;
      d[0] += bi * bi;
    }
    __syncthreads();
    cl_step<1>(d, cs, [&](const T (&s)[1]) {  // CgInit
      const T nrm = sqrt(s[0]);
      cs.nrhs2 = nrm * nrm;
      cs.rr = cs.nrhs2;
      cs.done = (cs.nrhs2 <= T(abs_tol * abs_tol)) ? kConverged : kRunning;
    });
    if (cs.done == kRunning) {
      T e[2] = {T(0), T(0)};
      for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
        const T acc = cl_row(A, r0 + i, sp, rank, shift);
        sq[i] = acc;
        e[0] += acc * acc;
        e[1] += sp[i] * acc;
      }
      cl_step<2>(e, cs, [&](const T (&s)[2]) {  // EpiCgFirst
        const T rr = cs.rr;
        const T alpha = rr / s[1];
        const T nap = sqrt(s[0]);
        cs.alpha = alpha;
        cs.beta = (alpha * alpha * nap * nap - rr) / rr;
        if (max_iters == 0) {
          cs.done = kMaxIters;
          cs.error = sqrt(fabs((double)rr) / (double)cs.nrhs2);
        }
      });
    }
    while (cs.done == kRunning) {
      const T alpha = cs.alpha, beta = cs.beta;
      T d1[1] = {T(0)};  // CgUpdate
      for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
        T vp = sp[i], vr = sr[i];
        sx[i] += alpha * vp;
        vr -= alpha * sq[i];
        vp = vr + beta * vp;
        d1[0] += vr * vr;
        sp[i] = vp;
        sr[i] = vr;
      }
      cl_step<1>(d1, cs, [&](const T (&s)[1]) { cs.rr = s[0]; });
      T e[2] = {T(0), T(0)};  // EpiCg
      for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
        const T acc = cl_row(A, r0 + i, sp, rank, shift);
        sq[i] = acc;
        e[0] += acc * acc;
        e[1] += sp[i] * acc;
      }
      cl_step<2>(e, cs, [&](const T (&s)[2]) {
        cs.iters += 1;
        const T rr = cs.rr;
        const double ratio = fabs((double)rr / (double)cs.nrhs2);
        if (ratio < tol * tol || fabs((double)rr) < abs_tol * abs_tol) {
          cs.done = kConverged;
          cs.error = sqrt(fabs((double)rr) / (double)cs.nrhs2);
          return;
        }
        const T a = rr / s[1];
        const T bb = (a * a * s[0] - rr) / rr;
        cs.alpha = a;
        cs.beta = bb;
        cs.error = sqrt(fabs((double)rr) / (double)cs.nrhs2);
        if (!finite_(a) || !finite_(bb)) cs.done = kBreakdown;
        else if (cs.iters >= max_iters) cs.done = kMaxIters;
      });
    }
  } else {
    T d[1] = {T(0)};  // PcgInit
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
      const T bi = b[r0 + i], di = dg[r0 + i];
      sd[i] = di;
      sx[i] = T(0); sr[i] = bi;
      const T zi = bi * di;
      sp[i] = zi;
      d[0] += bi * zi;
    }
    __syncthreads();
    cl_step<1>(d, cs, [&](const T (&s)[1]) {
      cs.ip = s[0];
      cs.nrhs2 = s[0];
      cs.done = (fabs((double)s[0]) <= abs_tol * abs_tol) ? kConverged : kRunning;
      if (cs.done == kRunning && max_iters == 0) cs.done = kMaxIters;
    });
    while (cs.done == kRunning) {
      T e[1] = {T(0)};  // EpiPcg
      for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
        const T acc = cl_row(A, r0 + i, sp, rank, shift);
        sq[i] = acc;
        e[0] += acc * sp[i];
      }
      cl_step<1>(e, cs, [&](const T (&s)[1]) {
        cs.iters += 1;
        cs.alpha = cs.ip / s[0];
        if (!finite_(cs.alpha)) cs.done = kBreakdown;
      });
      if (cs.done != kRunning) break;
      const T alpha = cs.alpha;
      T d1[1] = {T(0)};  // PcgUpdate (Jacobi)
      for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
        const T vp = sp[i];
        sx[i] += alpha * vp;
        const T vr = sr[i] - alpha * sq[i];
        sr[i] = vr;
        const T zi = vr * sd[i];
        sz[i] = zi;
        d1[0] += vr * zi;
      }
      cl_step<1>(d1, cs, [&](const T (&s)[1]) {  // pcg_check
        const T new_ip = s[0];
        const double ratio = (double)new_ip / (double)cs.nrhs2;
        cs.error = sqrt(fabs(ratio));
        if (fabs(ratio) < tol * tol || fabs((double)new_ip) < abs_tol * abs_tol) {
          cs.done = kConverged;
          return;
        }
        cs.beta = new_ip / cs.ip;
        cs.ip = new_ip;
        if (!finite_(cs.beta)) cs.done = kBreakdown;
        else if (cs.iters >= max_iters) cs.done = kMaxIters;
      });
      if (cs.done != kRunning) break;
      const T beta = cs.beta;
      for (uint32_t i = threadIdx.x; i < m; i += blockDim.x)  // PcgP
        sp[i] = sz[i] + beta * sp[i];
      cl_barrier();  // p complete in every CTA before the next product
    }
  }
  for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) x[r0 + i] = sx[i];
  if (rank == 0 && threadIdx.x == 0) {
    st->iters = cs.iters;
    st->error = cs.error;
    st->done = cs.done;
    st->rr = cs.rr;
  }
  // no CTA leaves while another may still read its shared memory
  cl_barrier();
}

// pipelined BiCGStab without a preconditioner (EpiBicgAp, BicgS, EpiBicgAs,
// BicgUpdate above) in one cluster; p and s are gathered by the products
template <typename T>
__global__ void __launch_bounds__(kClusterSolveThreads, 1)
    cluster_bicgstab_kernel(CsrView<T> A, const T *b, T *x, St<T> *st, uint32_t shift) {
  __shared__ ClState<T> cs;
  extern __shared__ __align__(16) unsigned char cl_vec_bytes[];
  cg::cluster_group cl = cg::this_cluster();
  const uint32_t rank = cl.block_rank(), len = 1u << shift;
  T *sx = reinterpret_cast<T *>(cl_vec_bytes), *sr = sx + len, *sp = sr + len, *sr0 = sp + len;
  T *sAp = sr0 + len, *ss = sAp + len, *sAs = ss + len;
  const uint32_t n = A.rows;
  const uint32_t r0 = min(rank << shift, n), r1 = min(r0 + len, n), m = r1 - r0;
  const double tol = st->tol, abs_tol = st->abs_tol;
  const unsigned max_iters = st->max_iters;
  if (threadIdx.x == 0) {
    cs.buf = 0;
    cs.iters = 0;
    cs.error = 0;
  }
  T d[1] = {T(0)};  // BicgInit
  for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
    const T bi = b[r0 + i];
    sx[i] = T(0); sr[i] = bi; sp[i] = bi; sr0[i] = bi;
    d[0] += bi * bi;
  }
  __syncthreads();
  cl_step<1>(d, cs, [&](const T (&v)[1]) {
    const T nrm = sqrt(v[0]);
    cs.nrhs = nrm;
    cs.r_r0 = nrm * nrm;
    cs.done = ((double)nrm <= abs_tol) ? kConverged : kRunning;
    if (cs.done == kRunning && max_iters == 0) { cs.done = kMaxIters; cs.error = 1.0; }
  });
  while (cs.done == kRunning) {
    T e[1] = {T(0)};  // EpiBicgAp
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
      const T acc = cl_row(A, r0 + i, sp, rank, shift);
      sAp[i] = acc;
      e[0] += acc * sr0[i];
    }
    cl_step<1>(e, cs, [&](const T (&v)[1]) {
      cs.iters += 1;
      cs.Ap_r0 = v[0];
      cs.alpha = cs.r_r0 / v[0];
    });
    const T alpha = cs.alpha;
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x)  // BicgS
      ss[i] = sr[i] - alpha * sAp[i];
    cl_barrier();  // s complete before the product gathers it
    // EpiBicgAs, with ||s||^2 (BicgS's reduction) from the same pass over s
    T g[4] = {T(0), T(0), T(0), T(0)};
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
      const T acc = cl_row(A, r0 + i, ss, rank, shift);
      const T vs = ss[i];
      sAs[i] = acc;
      g[0] += acc * acc;
      g[1] += vs * acc;
      g[2] += acc * sr0[i];
      g[3] += vs * vs;
    }
    cl_step<4>(g, cs, [&](const T (&v)[4]) {
      cs.s_s = v[3];
      const T a = cs.r_r0 / cs.Ap_r0;
      const T bb = -v[2] / cs.Ap_r0;
      const T w = v[1] / v[0];
      const T rn = sqrt(cs.s_s - T(2) * w * v[1] + w * w * v[0]);
      cs.alpha = a;
      cs.beta = bb;
      cs.omega = w;
      cs.error = (double)rn / (double)cs.nrhs;
      if (fabs((double)rn / (double)cs.nrhs) < tol || (double)rn < abs_tol) cs.done = kConverged;
      else if (!finite_(a) || !finite_(w) || !finite_(bb)) cs.done = kBreakdown;
    });
    if (cs.done != kRunning) break;  // converged before the x update, as bicgstab.hpp:197-198
    const T a = cs.alpha, w = cs.omega, bb = cs.beta;
    T h[1] = {T(0)};  // BicgUpdate
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
      T vp = sp[i];
      const T vs = ss[i];
      sx[i] += a * vp + w * vs;
      const T vr = vs - w * sAs[i];
      vp = vr + bb * (vp - w * sAp[i]);
      h[0] += vr * sr0[i];
      sr[i] = vr;
      sp[i] = vp;
    }
    cl_step<1>(h, cs, [&](const T (&v)[1]) {
      cs.r_r0 = v[0];
      if (cs.iters >= max_iters) cs.done = kMaxIters;
    });
  }
  for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) x[r0 + i] = sx[i];
  if (rank == 0 && threadIdx.x == 0) {
    st->iters = cs.iters;
    st->error = cs.error;
    st->done = cs.done;
    st->resnorm = cs.error * cs.nrhs;
  }
  cl_barrier();
}

// BiCGStab with a diagonal preconditioner (GbInit, EpiGbRestart<true>,
// EpiGb1, GbS, EpiGb2, GbUpdate, GbP above, bicgstab.hpp:398-489) in one
// cluster; products gather x (restarts), p and s
template <typename T>
__global__ void __launch_bounds__(kClusterSolveThreads, 1)
    cluster_gb_kernel(CsrView<T> A, const T *b, T *x, const T *dg, St<T> *st, uint32_t shift) {
  __shared__ ClState<T> cs;
  extern __shared__ __align__(16) unsigned char cl_vec_bytes[];
  cg::cluster_group cl = cg::this_cluster();
  const uint32_t rank = cl.block_rank(), len = 1u << shift;
  T *sx = reinterpret_cast<T *>(cl_vec_bytes), *sr = sx + len, *sp = sr + len, *sr0 = sp + len;
  T *st0 = sr0 + len, *ss = st0 + len, *st1 = ss + len, *sd = st1 + len;
  const uint32_t n = A.rows;
  const uint32_t r0 = min(rank << shift, n), r1 = min(r0 + len, n), m = r1 - r0;
  const double tol = st->tol, abs_tol = st->abs_tol;
  const unsigned max_iters = st->max_iters, max_before_restart = st->max_before_restart;
  if (threadIdx.x == 0) {
    cs.buf = 0;
    cs.iters = 0;
    cs.last_restart = 0;
    cs.error = 0;
  }
  T d[1] = {T(0)};  // GbInit
  for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
    const T bi = b[r0 + i];
    sx[i] = T(0);
    sd[i] = dg[r0 + i];
    d[0] += bi * bi;
  }
  __syncthreads();
  cl_step<1>(d, cs, [&](const T (&v)[1]) {
    const T nrm = sqrt(v[0]);
    cs.nrhs = nrm;
    cs.restart = 1;
    cs.done = ((double)nrm <= abs_tol) ? kConverged : kRunning;
    if (cs.done == kRunning && max_iters == 0) { cs.done = kMaxIters; cs.error = 1.0; }
  });
  while (cs.done == kRunning) {
    if (cs.restart) {
      T e[1] = {T(0)};  // EpiGbRestart (Jacobi): r = M^-1 (b - A x); p = r0* = r
      for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
        const T acc = cl_row(A, r0 + i, sx, rank, shift);
        const T v = (b[r0 + i] - acc) * sd[i];
        sp[i] = v;
        sr0[i] = v;
        sr[i] = v;
        e[0] += v * v;
      }
      cl_step<1>(e, cs, [&](const T (&v)[1]) {  // gb_restart_done
        const T nr = sqrt(v[0]);
        cs.ip = nr * nr;
        cs.restart = 0;
        cs.last_restart = cs.iters;
      });
    }
    T e1[1] = {T(0)};  // EpiGb1: t0 = M^-1 A p; <t0, r0*>
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
      const T v = cl_row(A, r0 + i, sp, rank, shift) * sd[i];
      st0[i] = v;
      e1[0] += v * sr0[i];
    }
    cl_step<1>(e1, cs, [&](const T (&v)[1]) {
      cs.iters += 1;
      cs.alpha = cs.ip / v[0];
    });
    const T alpha = cs.alpha;
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) ss[i] = sr[i] - alpha * st0[i];  // GbS
    cl_barrier();  // s complete in every CTA before its product
    T e2[2] = {T(0), T(0)};  // EpiGb2: t1 = M^-1 A s; ||t1||^2, <t1, s>
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
      const T v = cl_row(A, r0 + i, ss, rank, shift) * sd[i];
      st1[i] = v;
      e2[0] += v * v;
      e2[1] += v * ss[i];
    }
    cl_step<2>(e2, cs, [&](const T (&v)[2]) {  // gb_omega
      const T nt1 = sqrt(v[0]);
      cs.omega = v[1] / (nt1 * nt1);
    });
    const T a = cs.alpha, w = cs.omega;
    T e3[2] = {T(0), T(0)};  // GbUpdate
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
      const T vs = ss[i];
      sx[i] += a * sp[i] + w * vs;
      const T vr = vs - w * st1[i];
      sr[i] = vr;
      e3[0] += vr * vr;
      e3[1] += vr * sr0[i];
    }
    cl_step<2>(e3, cs, [&](const T (&v)[2]) {
      const T rn = sqrt(v[0]);
      cs.error = (double)rn / (double)cs.nrhs;
      if ((double)rn / (double)cs.nrhs < tol || (double)rn < abs_tol) {
        cs.done = kConverged;
        return;
      }
      const T new_ip = v[1];
      cs.beta = new_ip / cs.ip * cs.alpha / cs.omega;
      cs.ip = new_ip;
      const unsigned it = cs.iters - 1;
      if ((new_ip >= T(0) && new_ip <= T(0)) || (cs.omega >= T(0) && cs.omega <= T(0)) ||
          it - cs.last_restart > max_before_restart)
        cs.restart = 1;
      if (!finite_(cs.alpha) || !finite_(cs.omega)) cs.done = kBreakdown;
      else if (cs.iters >= max_iters) cs.done = kMaxIters;
    });
    if (cs.done != kRunning) break;
    const T bb = cs.beta, w2 = cs.omega;
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x)  // GbP
      sp[i] = sr[i] + bb * (sp[i] - w2 * st0[i]);
    cl_barrier();  // p (and x) complete before the next products
  }
  for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) x[r0 + i] = sx[i];
  if (rank == 0 && threadIdx.x == 0) {
    st->iters = cs.iters;
    st->error = cs.error;
    st->done = cs.done;
  }
  cl_barrier();
}

// CTAs of the small-system cluster the device can co-schedule (16, 8 or 4;
// 0: none), once per precision
template <typename T>
static int cluster_solve_ctas() {
  static std::atomic<int> cached{-1};
  int v = cached.load(std::memory_order_relaxed);
  if (v >= 0) return v;
  v = 0;
  auto k0 = cluster_cg_kernel<T, false>;
  auto k1 = cluster_cg_kernel<T, true>;
  auto k2 = cluster_bicgstab_kernel<T>;
  auto k3 = cluster_gb_kernel<T>;
  bool ok = cudaFuncSetAttribute(k3, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
                cudaSuccess &&
            cudaFuncSetAttribute(k3, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kClusterSolveSmem) == cudaSuccess &&
            cudaFuncSetAttribute(k2, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
                cudaSuccess &&
            cudaFuncSetAttribute(k2, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kClusterSolveSmem) == cudaSuccess &&
            cudaFuncSetAttribute(k0, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
                cudaSuccess &&
            cudaFuncSetAttribute(k1, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
                cudaSuccess &&
            cudaFuncSetAttribute(k0, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kClusterSolveSmem) == cudaSuccess &&
            cudaFuncSetAttribute(k1, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kClusterSolveSmem) == cudaSuccess;
  for (int cc : {16, 8, 4}) {
    if (!ok) break;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cc);
    cfg.blockDim = dim3(kClusterSolveThreads);
    cfg.dynamicSmemBytes = kClusterSolveSmem;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cc;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int c0 = 0, c1 = 0, c2 = 0, c3 = 0;
    if (cudaOccupancyMaxActiveClusters(&c0, k0, &cfg) == cudaSuccess && c0 > 0 &&
        cudaOccupancyMaxActiveClusters(&c1, k1, &cfg) == cudaSuccess && c1 > 0 &&
        cudaOccupancyMaxActiveClusters(&c2, k2, &cfg) == cudaSuccess && c2 > 0 &&
        cudaOccupancyMaxActiveClusters(&c3, k3, &cfg) == cudaSuccess && c3 > 0) {
      v = cc;
      break;
    }
  }
  (void)cudaGetLastError();
  cached.store(v, std::memory_order_relaxed);
  return v;
}

// Launch geometry of a small-system cluster solve: rows a CTA (a power of two
// covering n / cc, so a column's owner is a shift), threads a CTA (128, 256 or
// 512: a cluster barrier over fewer warps is quicker, measured best per size)
// and the shared memory of `vectors` slices; false if the solve does not
// apply (rows above the limit, more than kClusterSolveMaxChunk rows a CTA, not
// CSR, kernel timing on, no cluster, or the slices do not fit).
template <typename T>
static bool cluster_geometry(Backend &be, const Matrix &A, int vectors, int &cc, uint32_t &shift,
                             uint32_t &threads, size_t &smem) {
  const uint32_t n = A.rows;
  if (n == 0 || n > kClusterSolveMaxRows || A.format != VCLGB_CSR || be.timing) return false;
  cc = cluster_solve_ctas<T>();
  if (cc == 0) return false;
  shift = 5;
  while (((uint64_t)cc << shift) < n) ++shift;
  const uint32_t len = 1u << shift;
  if (len > kClusterSolveMaxChunk) return false;
  threads = len <= 128 ? 128 : len <= 256 ? 256 : kClusterSolveThreads;
  smem = (size_t)vectors * len * sizeof(T);
  return smem <= kClusterSolveSmem;
}

template <typename T, typename... KArgs, typename... Args>
static void cluster_launch(Backend &be, void (*kern)(KArgs...), int cc, uint32_t threads,
                           size_t smem, Args &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cc);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = be.stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = cc;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  VCLGB_CUDA(cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...));
  be.launches++;
}

// Runs the small-system CG (no preconditioner or a diagonal one) if it
// applies; false otherwise.
template <typename T>
static bool cluster_cg(Backend &be, const Matrix &A, const T *b, T *x, St<T> *st,
                       const Precond *P) {
  if (P && !diag_needed(P)) return false;
  int cc;
  uint32_t shift, threads;
  size_t smem;
  if (!cluster_geometry<T>(be, A, P ? 6 : 4, cc, shift, threads, smem)) return false;
  const CsrView<T> view{A.row_ptr, A.col_idx, static_cast<const T *>(A.values), A.rows};
  const T *dg = P ? P->inv_diag.as<T>() : nullptr;
  if (P)
    cluster_launch<T>(be, cluster_cg_kernel<T, true>, cc, threads, smem, view, b, x, dg, st, shift);
  else
    cluster_launch<T>(be, cluster_cg_kernel<T, false>, cc, threads, smem, view, b, x, dg, st,
                      shift);
  return true;
}

// Runs the small-system BiCGStab (pipelined without a preconditioner, or the
// preconditioned form with a diagonal one) if it applies; false otherwise.
template <typename T>
static bool cluster_bicgstab(Backend &be, const Matrix &A, const T *b, T *x, St<T> *st,
                             const Precond *P) {
  if (P && !diag_needed(P)) return false;
  int cc;
  uint32_t shift, threads;
  size_t smem;
  if (!cluster_geometry<T>(be, A, P ? 8 : 7, cc, shift, threads, smem)) return false;
  const CsrView<T> view{A.row_ptr, A.col_idx, static_cast<const T *>(A.values), A.rows};
  if (P)
    cluster_launch<T>(be, cluster_gb_kernel<T>, cc, threads, smem, view, b, x,
                      P->inv_diag.as<T>(), st, shift);
  else
    cluster_launch<T>(be, cluster_bicgstab_kernel<T>, cc, threads, smem, view, b, x, st, shift);
  return true;
}

// ---------------------------------------------------------------------------
// Unpreconditioned GMRES of a small system in one cluster: the per-phase
// solve's steps (GmInit, gm_cycle_check, GmScaleR, EpiGmResid, EpiGmV, the
// classical Gram-Schmidt pass, GmNormalize, GmCycleEnd, GmUpdateX) with x, r
// and the Krylov basis in shared memory, the products gathering through
// distributed shared memory.  The k dot products of a Gram-Schmidt step are
// summed in each CTA in chunks of eight, pushed to every CTA's slots and
// added after one cluster barrier; the other reductions are cl_step's.  Every
// CTA keeps the same GMRES state and runs the same scalar steps on thread 0.
// ---------------------------------------------------------------------------
constexpr uint32_t kClusterGmresMaxK = 32;

template <typename T>
struct GcState {
  ClState<T> cl;                        // single-value reductions (cl_step)
  T mpart[2][16][kClusterGmresMaxK];    // multi-dot slots by rank, double buffered
  T mwarp[8 * (kClusterSolveThreads / 32)];
  T nrhs, rho0, inv_rho0, rho, vnorm2, inv_vnorm;
  T R[kClusterGmresMaxK * kClusterGmresMaxK];
  T xi[kClusterGmresMaxK], h[kClusterGmresMaxK], coef[kClusterGmresMaxK];
  double tol, abs_tol, error;
  unsigned K, iters, restart_count, max_restarts;
  int kk, done, mbuf;
};

template <typename T>
__device__ __forceinline__ void gc_cycle_check(GcState<T> &g) {  // gm_cycle_check
  if ((double)g.rho0 <= g.abs_tol) { g.done = kConverged; return; }
  g.rho = T(1);
  if ((double)(g.rho0 / g.nrhs) < g.tol || (double)g.rho0 < g.abs_tol) {
    g.done = kConverged;
    return;
  }
  if (g.restart_count > g.max_restarts) g.done = kMaxIters;
}

template <typename T>
__device__ __forceinline__ void gc_cycle_end(GcState<T> &g) {  // GmCycleEnd
  if (g.done != kRunning) { g.kk = 0; return; }
  const unsigned K = g.K;
  unsigned k = K, full_k = K;
  for (unsigned i = 0; i < k; ++i)
    if (fabs((double)g.R[i + i * k]) < g.tol * (double)g.R[0]) { k = i; break; }
  T rho = g.rho;
  for (unsigned i = 0; i < k; ++i) {
    g.iters += 1;
    T xi = g.xi[i];
    if (xi >= rho || xi <= -rho) { k = i; break; }
    rho *= sin(acos(xi / rho));
  }
  g.rho = rho;
  T eta[kClusterGmresMaxK];
  for (unsigned i = 0; i < K; ++i) eta[i] = g.xi[i];
  for (int i2 = (int)k - 1; i2 > -1; --i2) {
    unsigned i = (unsigned)i2;
    for (unsigned j = i + 1; j < k; ++j) eta[i] -= g.R[i + j * full_k] * eta[j];
    eta[i] /= g.R[i + i * full_k];
  }
  for (unsigned i = 0; i < k; ++i) g.coef[i] = g.rho0 * eta[i];
  g.kk = (int)k;
  g.error = fabs((double)(rho * g.rho0 / g.nrhs));
  g.restart_count += 1;
}

// h_j = <v_j, w> for j < k over the cluster (V: columns of len entries);
// the sums land in g.h and in column k of R
template <typename T>
__device__ __forceinline__ void gc_multidot(const T *V, uint32_t len, const T *w, uint32_t m,
                                            uint32_t k, GcState<T> &g) {
  cg::cluster_group cl = cg::this_cluster();
  const unsigned nct = cl.num_blocks(), me = cl.block_rank();
  const int b = g.mbuf;
  for (uint32_t c0 = 0; c0 < k; c0 += 8) {
    T acc[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j] = T(0);
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
      const T wi = w[i];
#pragma unroll
      for (int j = 0; j < 8; ++j)
        if (c0 + j < k) acc[j] += V[(size_t)(c0 + j) * len + i] * wi;
    }
    block_sum<8>(acc, g.mwarp);  // valid in every lane of warp 0
    if (threadIdx.x < nct) {
      T *dst = cl.map_shared_rank(&g.mpart[b][me][c0], threadIdx.x);
#pragma unroll
      for (int j = 0; j < 8; ++j)
        if (c0 + j < k) dst[j] = acc[j];
    }
  }
  cl_barrier();
  if (threadIdx.x < 32) {
    for (uint32_t j = threadIdx.x; j < k; j += 32) {
      T t = T(0);
      for (unsigned r = 0; r < nct; ++r) t += g.mpart[b][r][j];
      g.h[j] = t;
      g.R[j + (size_t)k * g.K] = t;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) g.mbuf = b ^ 1;
}

template <typename T>
__global__ void __launch_bounds__(kClusterSolveThreads, 1)
    cluster_gmres_kernel(CsrView<T> A, const T *b, T *x, Gm<T> *gout, uint32_t shift) {
  __shared__ GcState<T> g;
  extern __shared__ __align__(16) unsigned char cl_vec_bytes[];
  cg::cluster_group cl = cg::this_cluster();
  const uint32_t rank = cl.block_rank(), len = 1u << shift;
  T *sx = reinterpret_cast<T *>(cl_vec_bytes), *sr = sx + len, *sV = sr + len;
  const uint32_t n = A.rows;
  const uint32_t r0 = min(rank << shift, n), r1 = min(r0 + len, n), m = r1 - r0;
  const uint32_t K = gout->K;
  if (threadIdx.x == 0) {
    g.cl.buf = 0;
    g.mbuf = 0;
    g.K = K;
    g.tol = gout->tol;
    g.abs_tol = gout->abs_tol;
    g.max_restarts = gout->max_restarts;
  }
  T d[1] = {T(0)};  // GmInit
  for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
    const T bi = b[r0 + i];
    sx[i] = T(0);
    sr[i] = bi;
    d[0] += bi * bi;
  }
  __syncthreads();
  cl_step<1>(d, g.cl, [&](const T (&s)[1]) {
    g.nrhs = sqrt(s[0]);
    g.rho0 = g.nrhs;
    g.inv_rho0 = T(1) / g.rho0;
    g.rho = T(1);
    g.iters = 0;
    g.error = 0;
    g.restart_count = 0;
    g.done = kRunning;
    gc_cycle_check(g);  // GmCheckFirst
  });
  {
    const T inv = g.inv_rho0;  // GmScaleR
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) sr[i] *= inv;
  }
  cl_barrier();  // r complete before the first product gathers it
  bool first = true;
  while (g.done == kRunning) {
    if (!first) {
      T e[1] = {T(0)};  // EpiGmResid: r = b - A x
      for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
        const T v = b[r0 + i] - cl_row(A, r0 + i, sx, rank, shift);
        sr[i] = v;
        e[0] += v * v;
      }
      cl_step<1>(e, g.cl, [&](const T (&s)[1]) {
        g.rho0 = sqrt(s[0]);
        g.inv_rho0 = T(1) / g.rho0;
        gc_cycle_check(g);
      });
      if (g.done != kRunning) break;
      const T inv = g.inv_rho0;  // GmScaleR
      for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) sr[i] *= inv;
      cl_barrier();
    }
    first = false;
    for (uint32_t k = 0; k < K; ++k) {
      T *vk = sV + (size_t)k * len;
      const T *src = k == 0 ? sr : sV + (size_t)(k - 1) * len;
      // v_k = A src; for k = 0 ||v_k||^2 and <r, v_k> come with it (EpiGmV)
      T e[2] = {T(0), T(0)};
      for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
        const T acc = cl_row(A, r0 + i, src, rank, shift);
        vk[i] = acc;
        e[0] += acc * acc;
        e[1] += sr[i] * acc;
      }
      if (k > 0) {  // classical Gram-Schmidt against v_0 .. v_{k-1}: w, ||w||^2, <r, w>
        gc_multidot(sV, len, vk, m, k, g);
        e[0] = e[1] = T(0);
        for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
          T w = vk[i];
          for (uint32_t j = 0; j < k; ++j) w -= g.h[j] * sV[(size_t)j * len + i];
          vk[i] = w;
          e[0] += w * w;
          e[1] += sr[i] * w;
        }
      }
      // GmNormalize from the same reduction: R(k,k) = ||w||, xi_k = <r, w> / ||w||,
      // then v_k /= ||w|| on this CTA's rows and a barrier before the next
      // product gathers them
      cl_step<2>(e, g.cl, [&](const T (&s)[2]) {
        g.vnorm2 = s[0];
        g.inv_vnorm = T(1) / sqrt(s[0]);
        g.xi[k] = s[1] * g.inv_vnorm;
        g.R[k + (size_t)k * g.K] = sqrt(s[0]);
      });
      const T nv = g.inv_vnorm;
      for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) vk[i] *= nv;
      cl_barrier();
    }
    if (threadIdx.x == 0) gc_cycle_end(g);
    __syncthreads();
    if (g.done == kRunning && g.kk > 0) {  // GmUpdateX
      const int kk = g.kk;
      for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
        T v = sx[i] + g.coef[0] * sr[i];
        for (int j = 1; j < kk; ++j) v += g.coef[j] * sV[(size_t)(j - 1) * len + i];
        sx[i] = v;
      }
    }
    cl_barrier();  // x complete before the next residual product gathers it
  }
  for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) x[r0 + i] = sx[i];
  if (rank == 0 && threadIdx.x == 0) {
    gout->iters = g.iters;
    gout->error = g.error;
    gout->done = g.done;
  }
  cl_barrier();  // no CTA leaves while another may still read its shared memory
}

// CTAs of the small-system GMRES cluster (16, 8 or 4; 0: none), once per precision
template <typename T>
static int cluster_gmres_ctas() {
  static std::atomic<int> cached{-1};
  int v = cached.load(std::memory_order_relaxed);
  if (v >= 0) return v;
  v = 0;
  auto k = cluster_gmres_kernel<T>;
  const bool ok =
      cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess &&
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)kClusterSolveSmem) == cudaSuccess;
  for (int cc : {16, 8, 4}) {
    if (!ok) break;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cc);
    cfg.blockDim = dim3(kClusterSolveThreads);
    cfg.dynamicSmemBytes = kClusterSolveSmem;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cc;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int c = 0;
    if (cudaOccupancyMaxActiveClusters(&c, k, &cfg) == cudaSuccess && c > 0) {
      v = cc;
      break;
    }
  }
  (void)cudaGetLastError();
  cached.store(v, std::memory_order_relaxed);
  return v;
}

// Runs the unpreconditioned small-system GMRES if it applies (Krylov
// dimension at most 32, x, r and the basis fit the CTAs' shared memory);
// false otherwise.  g holds the solve's parameters and receives its outcome.
template <typename T>
static bool cluster_gmres(Backend &be, const Matrix &A, const T *b, T *x, Gm<T> *g,
                          uint32_t K) {
  if (K > kClusterGmresMaxK) return false;
  const uint32_t n = A.rows;
  if (n == 0 || n > kClusterSolveMaxRows || A.format != VCLGB_CSR || be.timing) return false;
  const int cc = cluster_gmres_ctas<T>();
  if (cc == 0) return false;
  uint32_t shift = 5;
  while (((uint64_t)cc << shift) < n) ++shift;
  const uint32_t len = 1u << shift;
  if (len > kClusterSolveMaxChunk) return false;
  const size_t smem = (size_t)(K + 2) * len * sizeof(T);
  if (smem > kClusterSolveSmem) return false;
  const uint32_t threads = len <= 128 ? 128 : len <= 256 ? 256 : kClusterSolveThreads;
  const CsrView<T> view{A.row_ptr, A.col_idx, static_cast<const T *>(A.values), A.rows};
  cluster_launch<T>(be, cluster_gmres_kernel<T>, cc, threads, smem, view, b, x, g, shift);
  return true;
}

// bytes a product streams from the matrix (indices, values, row pointers)
static inline size_t matrix_stream_bytes(const Matrix &A) {
  return (size_t)A.nnz * (4 + A.vsize()) + ((size_t)A.rows + 1) * 4;
}

// Whether the solver's vectors go into the L2 window: where the products
// gather only near each row (stencils: CSR rows in one length bin, or the DIA
// form), the vectors an iteration writes and re-reads from HBM are the traffic
// the window saves (Jacobi-PCG on 192^3 diffusion 363 -> 253 us an iteration,
// CG on 128^3 75.3 -> 69.5).  Products that gather at random over the whole
// vector (irregular rows) already find most of it in L2, and the set-aside
// left the rest too little (BiCGStab on the 4M-row lognormal matrix 1076 ->
// 1354 us an iteration).
static inline bool l2_window_pays(const Matrix &A0) {
  const Matrix &A = spmv_form(A0);
  return (A.format == VCLGB_CSR && A.num_bins == 1 && A.bins[0].identity) ||
         A.format == kFormatDia;
}

template <typename T>
void cg_solve(Backend &be, Matrix &A, const T *b, T *x, vclgbSolverTag *tag, const Precond *P) {
  const uint32_t n = A.rows;
  require(A.rows == A.cols, VCLGB_INVALID_ARGUMENT, "CG needs a square matrix");
  Workspace ws;
  size_t o_st = ws.add(sizeof(St<T>));
  size_t o_part = ws.add(8 * kMaxSpmvGrid * sizeof(T));
  size_t o_cnt = ws.add(64);
  size_t vb = std::max<size_t>(n, 1) * sizeof(T);
  // the vectors of an iteration as one range for the L2 window, the gathered
  // p first (a window is at most 128 MB), then x's working copy
  size_t o_p = ws.add(vb), o_x = ws.add(vb);
  size_t o_r = ws.add(vb), o_q = ws.add(vb), o_z = ws.add(vb);
  size_t o_hyb = ws.add(hyb_scratch_bytes(A));
  ws.commit(be);
  St<T> *st = ws.at<St<T>>(o_st);
  St<T> h0 = make_state<T>(tag);
  VCLGB_CUDA(cudaMemcpyAsync(st, &h0, sizeof(h0), cudaMemcpyHostToDevice, be.stream));
  Reduction red{ws.at<void>(o_part), ws.at<unsigned>(o_cnt)};
  T *r = ws.at<T>(o_r), *p = ws.at<T>(o_p), *q = ws.at<T>(o_q), *z = ws.at<T>(o_z);
  void *hyb = ws.at<void>(o_hyb);
  const int *done = &st->done;
  uint32_t every = auto_check_every(tag, n);
  uint32_t chunks = tag->max_iters / every + 2;

  if (cluster_cg<T>(be, A, b, x, st, P)) {
    set_tag_outputs(be, st, tag);
    return;
  }
  // x, r, p, q (and z with a preconditioner) kept in L2 while A streams:
  // the iterations update the working copy of x, copied out at the end
  T *const x_out = x;
  const size_t vec_bytes = (size_t)((char *)((P ? z : q) + n) - (char *)p);
  L2Persist l2(be, p, l2_window_pays(A) ? vec_bytes : 0, matrix_stream_bytes(A));
  if (l2.on) x = ws.at<T>(o_x);
  if (!P) {
    // pipelined CG
    vec_pass<T>(be, n, CgInit<T>{b, x, r, p, st}, red);
    spmv_launch<T>(be, A, p, 0, 1, EpiCgFirst<T>{q, p, st}, red, q, 0, 1, T(1), T(0), done, hyb);
    run_iterations(be, done, chunks, every, true, [&]() {
      vec_pass<T>(be, n, CgUpdate<T>{x, p, r, q, st}, red);
      spmv_launch<T>(be, A, p, 0, 1, EpiCg<T>{q, p, st}, red, q, 0, 1, T(1), T(0), done, hyb);
    });
  } else {
    const bool jac = diag_needed(P);
    const T *dg = jac ? P->inv_diag.as<T>() : nullptr;  // 1 / diag
    if (jac) {
      vec_pass<T>(be, n, PcgInit<T, true>{b, dg, x, r, z, p, st}, red);
    } else {
      vec_pass<T>(be, n, PcgInit<T, false>{b, dg, x, r, z, p, st}, red);
      precond_apply(be, *P, z, nullptr);
      vec_pass<T>(be, n, PcgInitFinish<T>{r, z, p, st}, red);
    }
    run_iterations(be, done, chunks, every, true, [&]() {
      spmv_launch<T>(be, A, p, 0, 1, EpiPcg<T>{q, p, st}, red, q, 0, 1, T(1), T(0), done, hyb);
      if (jac)
        vec_pass<T>(be, n, PcgUpdate<T, true>{x, r, z, p, q, dg, st}, red);
      else
        vec_pass<T>(be, n, PcgUpdate<T, false>{x, r, z, p, q, dg, st}, red);
      if (!jac) {
        precond_apply(be, *P, z, done);
        vec_pass<T>(be, n, PcgDot<T>{r, z, st}, red);
      }
      vec_pass<T>(be, n, PcgP<T>{p, z, st}, red);
    });
  }
  if (x != x_out)
    VCLGB_CUDA(cudaMemcpyAsync(x_out, x, (size_t)n * sizeof(T), cudaMemcpyDeviceToDevice,
                               be.stream));
  set_tag_outputs(be, st, tag);
}

template <typename T>
void bicgstab_solve(Backend &be, Matrix &A, const T *b, T *x, vclgbSolverTag *tag,
                    const Precond *P) {
  const uint32_t n = A.rows;
  require(A.rows == A.cols, VCLGB_INVALID_ARGUMENT, "BiCGStab needs a square matrix");
  Workspace ws;
  size_t o_st = ws.add(sizeof(St<T>));
  size_t o_part = ws.add(8 * kMaxSpmvGrid * sizeof(T));
  size_t o_cnt = ws.add(64);
  size_t vb = std::max<size_t>(n, 1) * sizeof(T);
  // the vectors of an iteration as one range for the L2 window: the gathered
  // p and s first (a window is at most 128 MB), then x's working copy
  size_t o_p = ws.add(vb), o_s = ws.add(vb), o_x = ws.add(vb), o_r = ws.add(vb),
         o_r0 = ws.add(vb), o_Ap = ws.add(vb), o_As = ws.add(vb);
  size_t o_hyb = ws.add(hyb_scratch_bytes(A));
  ws.commit(be);
  St<T> *st = ws.at<St<T>>(o_st);
  St<T> h0 = make_state<T>(tag);
  VCLGB_CUDA(cudaMemcpyAsync(st, &h0, sizeof(h0), cudaMemcpyHostToDevice, be.stream));
  Reduction red{ws.at<void>(o_part), ws.at<unsigned>(o_cnt)};
  T *r = ws.at<T>(o_r), *p = ws.at<T>(o_p), *r0 = ws.at<T>(o_r0), *Ap = ws.at<T>(o_Ap),
    *s = ws.at<T>(o_s), *As = ws.at<T>(o_As);
  void *hyb = ws.at<void>(o_hyb);
  const int *done = &st->done;
  uint32_t every = auto_check_every(tag, n);
  uint32_t chunks = tag->max_iters / every + 2;

  if (cluster_bicgstab<T>(be, A, b, x, st, P)) {
    set_tag_outputs(be, st, tag);
    return;
  }
  // the vectors kept in L2 while A streams; the iterations update the working
  // copy of x, copied out at the end
  T *const x_out = x;
  L2Persist l2(be, p, l2_window_pays(A) ? (size_t)((char *)(As + n) - (char *)p) : 0,
               matrix_stream_bytes(A));
  if (l2.on) x = ws.at<T>(o_x);
  if (!P) {
    vec_pass<T>(be, n, BicgInit<T>{b, x, r, p, r0, st}, red);
    run_iterations(be, done, chunks, every, true, [&]() {
      spmv_launch<T>(be, A, p, 0, 1, EpiBicgAp<T>{Ap, r0, st}, red, Ap, 0, 1, T(1), T(0), done, hyb);
      vec_pass<T>(be, n, BicgS<T>{s, r, Ap, st}, red);
      spmv_launch<T>(be, A, s, 0, 1, EpiBicgAs<T>{As, s, r0, st}, red, As, 0, 1, T(1), T(0), done, hyb);
      vec_pass<T>(be, n, BicgUpdate<T>{x, p, r, s, As, Ap, r0, st}, red);
    });
  } else {
    const bool jac = diag_needed(P);
    const T *dg = jac ? P->inv_diag.as<T>() : nullptr;  // 1 / diag
    // t0 -> Ap, t1 -> As
    vec_pass<T>(be, n, GbInit<T>{b, x, st}, red);
    const int *rskip = &st->restart_skip;
    run_iterations(be, done, chunks, every, true, [&]() {
      if (jac)
        spmv_launch<T>(be, A, x, 0, 1, EpiGbRestart<T, true>{r, p, r0, b, dg, st}, red, r, 0, 1,
                       T(1), T(0), rskip, hyb);
      else
        spmv_launch<T>(be, A, x, 0, 1, EpiGbRestart<T, false>{r, p, r0, b, dg, st}, red, r, 0,
                       1, T(1), T(0), rskip, hyb);
      if (!jac) {
        precond_apply(be, *P, r, rskip);
        vec_pass<T>(be, n, GbRestartFinish<T>{p, r0, r, st}, red);
        spmv_launch<T>(be, A, p, 0, 1, EpiStore<T>{Ap, done}, red, Ap, 0, 1, T(1), T(0), done, hyb);
        precond_apply(be, *P, Ap, done);
        vec_pass<T>(be, n, GbDot1<T>{Ap, r0, st}, red);
      } else {
        spmv_launch<T>(be, A, p, 0, 1, EpiGb1<T>{Ap, dg, r0, st}, red, Ap, 0, 1, T(1), T(0), done, hyb);
      }
      vec_pass<T>(be, n, GbS<T>{s, r, Ap, st}, red);
      if (!jac) {
        spmv_launch<T>(be, A, s, 0, 1, EpiStore<T>{As, done}, red, As, 0, 1, T(1), T(0), done, hyb);
        precond_apply(be, *P, As, done);
        vec_pass<T>(be, n, GbDot2<T>{As, s, st}, red);
      } else {
        spmv_launch<T>(be, A, s, 0, 1, EpiGb2<T>{As, dg, s, st}, red, As, 0, 1, T(1), T(0), done, hyb);
      }
      vec_pass<T>(be, n, GbUpdate<T>{x, r, p, s, As, r0, st}, red);
      vec_pass<T>(be, n, GbP<T>{p, r, Ap, st}, red);
    });
  }
  if (x != x_out)
    VCLGB_CUDA(cudaMemcpyAsync(x_out, x, (size_t)n * sizeof(T), cudaMemcpyDeviceToDevice,
                               be.stream));
  set_tag_outputs(be, st, tag);
}

template <typename T>
static void gmres_pipelined_solve(Backend &be, Matrix &A, const T *b, T *x, vclgbSolverTag *tag) {
  const uint32_t n = A.rows;
  const uint32_t K = tag->krylov_dim ? tag->krylov_dim : 20;
  require(A.rows == A.cols, VCLGB_INVALID_ARGUMENT, "GMRES needs a square matrix");
  require(K <= (uint32_t)kGmresMaxK, VCLGB_INVALID_ARGUMENT, "krylov_dim must be <= 64");
  Workspace ws;
  size_t o_g = ws.add(sizeof(Gm<T>));
  size_t o_part = ws.add((size_t)kGmresMaxK * kMaxSpmvGrid * sizeof(T));
  size_t o_cnt = ws.add(64);
  size_t ld = ((size_t)std::max<uint32_t>(n, 1) + 31) / 32 * 32;
  size_t o_r = ws.add(ld * sizeof(T));
  size_t o_V = ws.add(ld * K * sizeof(T));
  size_t o_hyb = ws.add(hyb_scratch_bytes(A));
  ws.commit(be);
  Gm<T> *g = ws.at<Gm<T>>(o_g);
  {
    Gm<T> h;
    std::memset(&h, 0, sizeof(h));
    h.K = K;
    h.tol = tag->tol;
    h.abs_tol = tag->abs_tol;
    unsigned mr = tag->max_iters / K;
    if (mr > 0 && mr * K == tag->max_iters) mr -= 1;  // gmres_tag::max_restarts
    h.max_restarts = mr;
    VCLGB_CUDA(cudaMemcpyAsync(g, &h, sizeof(h), cudaMemcpyHostToDevice, be.stream));
  }
  Reduction red{ws.at<void>(o_part), ws.at<unsigned>(o_cnt)};
  T *r = ws.at<T>(o_r), *V = ws.at<T>(o_V);
  void *hyb = ws.at<void>(o_hyb);
  const int *done = &g->done;
  auto read_outcome = [&]() {
    Gm<T> h;
    VCLGB_CUDA(cudaMemcpyAsync(&h, g, sizeof(h), cudaMemcpyDeviceToHost, be.stream));
    VCLGB_CUDA(cudaStreamSynchronize(be.stream));
    tag->iters = h.iters;
    tag->error = h.error;
    tag->status = h.done == kConverged ? VCLGB_SUCCESS
                : h.done == kMaxIters  ? VCLGB_NOT_CONVERGED
                                       : VCLGB_BREAKDOWN;
  };
  if (cluster_gmres<T>(be, A, b, x, g, K)) {
    read_outcome();
    return;
  }
  vec_pass<T>(be, n, GmInit<T>{b, x, r, g}, red);
  scalar_step(be, GmCheckFirst<T>{g});
  vec_pass<T>(be, n, GmScaleR<T>{r, g}, red);
  bool first = true;
  auto cycle = [&]() {
    if (!first) {
      spmv_launch<T>(be, A, x, 0, 1, EpiGmResid<T>{r, b, g}, red, r, 0, 1, T(1), T(0), done, hyb);
      vec_pass<T>(be, n, GmScaleR<T>{r, g}, red);
    }
    for (uint32_t k = 0; k < K; ++k) {
      T *vk = V + (size_t)k * ld;
      const T *src = k == 0 ? r : V + (size_t)(k - 1) * ld;
      if (k == 0)
        spmv_launch<T>(be, A, src, 0, 1, EpiGmV<T>{vk, r, g}, red, vk, 0, 1, T(1), T(0), done,
                       hyb);
      else
        spmv_launch<T>(be, A, src, 0, 1, EpiGmVStore<T>{vk, g}, red, vk, 0, 1, T(1), T(0), done,
                       hyb);
      if (k > 0)
        cgs_pass<T>(be, n, (int)k, V, ld, vk, GmDots<T>{g, (int)k}, GmOrthEnd<T>{g, r, (int)k},
                    static_cast<T *>(red.partials), red.counter);
      vec_pass<T>(be, n, GmNormalize<T>{vk, g}, red);
    }
    scalar_step(be, GmCycleEnd<T>{g});
    vec_pass<T>(be, n, GmUpdateX<T>{x, r, V, ld, g}, red);
  };
  // first cycle (no residual recomputation), then captured cycles
  cycle();
  first = false;
  uint32_t max_cycles = tag->max_iters / K + 3;
  run_iterations(be, done, max_cycles, 1, true, cycle);
  read_outcome();
}

// linalg::solve(A, b, gmres_tag, precond) with any preconditioner
// (gmres.hpp:449-631); see Gh above.  Jacobi and row scaling are fused into
// the SpMV epilogues as a multiplication by the reciprocal diagonal; any
// other preconditioner runs between the kernels.
template <typename T>
static void gmres_precond_solve(Backend &be, Matrix &A, const T *b, T *x, vclgbSolverTag *tag,
                                const Precond *P) {
  const uint32_t n = A.rows;
  uint32_t K = tag->krylov_dim ? tag->krylov_dim : 20;
  require(K <= (uint32_t)kGmresMaxK, VCLGB_INVALID_ARGUMENT, "krylov_dim must be <= 64");
  if (n < K) K = n;  // gmres.hpp:466-468
  if (K == 0) K = 1;
  const bool jac = diag_needed(P);
  Workspace ws;
  size_t o_g = ws.add(sizeof(Gh<T>));
  size_t o_part = ws.add((size_t)kGmresMaxK * kMaxSpmvGrid * sizeof(T));
  size_t o_cnt = ws.add(64);
  const size_t ld = ((size_t)std::max<uint32_t>(n, 1) + 31) / 32 * 32;
  size_t o_r = ws.add(ld * sizeof(T)), o_w = ws.add(ld * sizeof(T));
  size_t o_Q = ws.add(ld * K * sizeof(T));
  size_t o_hyb = ws.add(hyb_scratch_bytes(A));
  ws.commit(be);
  Gh<T> *g = ws.at<Gh<T>>(o_g);
  {
    Gh<T> h;
    std::memset(&h, 0, sizeof(h));
    h.K = K;
    h.tol = tag->tol;
    h.abs_tol = tag->abs_tol;
    // gmres_tag::max_restarts (gmres.hpp:74-80) from the tag's krylov_dim
    const uint32_t kd = tag->krylov_dim ? tag->krylov_dim : 20;
    unsigned mr = tag->max_iters / kd;
    if (mr > 0 && mr * kd == tag->max_iters) mr -= 1;
    h.max_restarts = mr;
    VCLGB_CUDA(cudaMemcpyAsync(g, &h, sizeof(h), cudaMemcpyHostToDevice, be.stream));
  }
  Reduction red{ws.at<void>(o_part), ws.at<unsigned>(o_cnt)};
  T *r = ws.at<T>(o_r), *w = ws.at<T>(o_w), *Q = ws.at<T>(o_Q);
  const T *inv_d = jac ? P->inv_diag.as<T>() : nullptr;  // formed with the preconditioner
  void *hyb = ws.at<void>(o_hyb);
  const int *done = &g->done, *sskip = &g->step_skip;
  vec_pass<T>(be, n, GhInit<T>{b, x, g}, red);
  T *part = static_cast<T *>(red.partials);
  auto cycle = [&]() {
    // r = M^-1 (b - A x), rho_0, the restart test, r /= rho_0
    if (jac) {
      spmv_launch<T>(be, A, x, 0, 1, EpiGhResid<T, true>{r, b, inv_d, g}, red, r, 0, 1, T(1),
                     T(0), done, hyb);
    } else {
      spmv_launch<T>(be, A, x, 0, 1, EpiGhResid<T, false>{r, b, inv_d, g}, red, r, 0, 1, T(1),
                     T(0), done, hyb);
      precond_apply(be, *P, r, done);
      vec_pass<T>(be, n, GhResidNorm<T>{r, g}, red);
    }
    vec_pass<T>(be, n, GhScaleR<T>{r, g}, red);
    for (uint32_t k = 0; k < K; ++k) {
      const T *src = k == 0 ? r : Q + (size_t)(k - 1) * ld;
      // the step's test runs in the last reduction over w: the product's (or
      // the norm pass's) at k = 0, the last Gram-Schmidt pass's after
      if (jac && k == 0) {
        spmv_launch<T>(be, A, src, 0, 1, EpiGhW<T, true, true>{w, inv_d, r, g}, red, w, 0, 1,
                       T(1), T(0), sskip, hyb);
      } else if (jac) {
        spmv_launch<T>(be, A, src, 0, 1, EpiGhW<T, true, false>{w, inv_d, r, g}, red, w, 0, 1,
                       T(1), T(0), sskip, hyb);
      } else {
        spmv_launch<T>(be, A, src, 0, 1, EpiGhW<T, false, false>{w, inv_d, r, g}, red, w, 0, 1,
                       T(1), T(0), sskip, hyb);
        precond_apply(be, *P, w, sskip);
        if (k == 0) vec_pass<T>(be, n, GhWNorm<T, true>{w, r, g}, red);
        else vec_pass<T>(be, n, GhWNorm<T, false>{w, r, g}, red);
      }
      if (k > 0) {
        cgs_pass<T>(be, n, (int)k, Q, ld, w, GhDots<T, false>{g, (int)k},
                    GhOrthEnd<T, false>{g, r, (int)k}, part, red.counter);
        cgs_pass<T>(be, n, (int)k, Q, ld, w, GhDots<T, true>{g, (int)k},
                    GhOrthEnd<T, true>{g, r, (int)k}, part, red.counter);
      }
      vec_pass<T>(be, n, GhNormalize<T>{Q + (size_t)k * ld, w, g, (int)k}, red);
    }
    scalar_step(be, GhCycleEnd<T>{g});
    vec_pass<T>(be, n, GhUpdateX<T>{x, r, Q, ld, g}, red);
    scalar_step(be, GhCycleClose<T>{g});
  };
  const uint32_t max_cycles = tag->max_iters / std::max<uint32_t>(K, 1) + 3;
  run_iterations(be, done, max_cycles, 1, true, cycle);
  Gh<T> h;
  VCLGB_CUDA(cudaMemcpyAsync(&h, g, sizeof(h), cudaMemcpyDeviceToHost, be.stream));
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  tag->iters = h.iters;
  tag->error = h.error;
  tag->status = h.done == kConverged ? VCLGB_SUCCESS
              : h.done == kMaxIters  ? VCLGB_NOT_CONVERGED
                                     : VCLGB_BREAKDOWN;
}

template <typename T>
void gmres_solve(Backend &be, Matrix &A, const T *b, T *x, vclgbSolverTag *tag,
                 const Precond *P) {
  require(A.rows == A.cols, VCLGB_INVALID_ARGUMENT, "GMRES needs a square matrix");
  if (P) gmres_precond_solve<T>(be, A, b, x, tag, P);
  else gmres_pipelined_solve<T>(be, A, b, x, tag);
}

}  // namespace vclgb

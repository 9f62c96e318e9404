// Per-compartment cell physics of the four cerebellar cell types: gating
// updates (the reference's *_update_ion_RKC kernels), Ca dynamics, Nernst
// potentials and the frozen current vector b (the *_update_matrix kernels).
//
// Templated on the gating type R: R = double gives the plain FP64 path, whose
// expressions keep the reference's operation order (this file is compiled
// with -fmad=false and uses the canonical exp/log, so it matches the oracle's
// canonical mode bit for bit); R = float gives the mixed path (FP32 gating,
// channel currents and b accumulation).  Calcium, reversal potentials and
// the arguments of the discontinuous functions (the Purkinje Ca quantisation,
// the Kdr tau step, the HCN2 ramp) stay FP64 in both.
//
// Reference: pkj_ion.cu:4-91,304-358; io_ion.cu:5-51,91-126; gr_ion.cu:3-207,
// 461-480; go_ion.cu:3-213,379-437; solve_rkc.cu:227-435 (b assembly).
#pragma once
#include "canon_math.cuh"
#include "model.h"

namespace gbrkc {

__device__ __forceinline__ double mexp(double x) { return cm_exp(x); }
__device__ __forceinline__ float mexp(float x) { return expf(x); }
__device__ __forceinline__ double mlog(double x) { return cm_log(x); }
__device__ __forceinline__ float mlog(float x) { return logf(x); }
__device__ __forceinline__ double mabs(double x) { return fabs(x); }
__device__ __forceinline__ float mabs(float x) { return fabsf(x); }
__device__ __forceinline__ double mmin(double a, double b) { return fmin(a, b); }
__device__ __forceinline__ float mmin(float a, float b) { return fminf(a, b); }

// c * x / (1 - exp(-x / k)), the form of many Hodgkin-Huxley rate functions,
// with a removable singularity at x = 0 (limit c * k).  FP64 evaluates the
// reference's expression as written (the voltage would have to hit the
// singular point exactly).  FP32 gating rounds the voltage to float first, so
// x = 0 comes up about 10^8 times more often (0 / 0 = NaN stops the cell);
// there, for |x / k| < 1e-3, the series c k (1 + u/2 + u^2/12), u = x / k, is
// used instead -- the guard NEURON's hh.mod applies in its vtrap function.
template <typename R>
__device__ __forceinline__ R hh_xr(R c, R x, R k) {
  if constexpr (sizeof(R) == 4) {
    const R u = x / k;
    if (mabs(u) < R(1e-3)) return c * k * (R(1) + u * (R(0.5) + u * R(1.0 / 12.0)));
  }
  return c * x / (R(1) - mexp(-x / k));
}

// trapezoid gate step of every RKC ion kernel: (2 dt x_inf + (2 tau - dt) x) / (2 tau + dt)
template <typename R>
__device__ __forceinline__ R trap(R dt, R inf, R tau, R x) {
  return (R(2.0) * dt * inf + (R(2.0) * tau - dt) * x) / (R(2.0) * tau + dt);
}

// View of one compartment's gate and conductance slots in a pool (SoA).
template <typename R>
struct Slots {
  R *ion;
  const R *cond;
  long stride;
  long i;
  __device__ R &x(int k) const { return ion[(long)k * stride + i]; }
  __device__ R g(int k) const { return cond[(long)k * stride + i]; }
};

// ---------------------------------------------------------------- Purkinje
template <typename R> struct Pkj {
  __device__ static R l(R v, R A, R B, R C, R D) { return A / (B + mexp((v + C) / D)); }
  __device__ static R am_NaF(R v) { return l(v, R(35.0), R(0.0), R(5.0), R(-10.0)); }
  __device__ static R ah_NaF(R v) { return l(v, R(0.225), R(1.0), R(80.0), R(10.0)); }
  __device__ static R am_NaP(R v) { return l(v, R(200.0), R(1.0), R(-18.0), R(-16.0)); }
  __device__ static R am_CaP(R v) { return l(v, R(8.5), R(1.0), R(-8.0), R(-12.5)); }
  __device__ static R ah_CaP(R v) { return l(v, R(0.0015), R(1.0), R(29.0), R(8.0)); }
  __device__ static R am_CaT(R v) { return l(v, R(2.60), R(1.0), R(21.0), R(-8.0)); }
  __device__ static R ah_CaT(R v) { return l(v, R(0.0025), R(1.0), R(40.0), R(8.0)); }
  __device__ static R am_KA(R v) { return l(v, R(1.40), R(1.0), R(27.0), R(-12.0)); }
  __device__ static R ah_KA(R v) { return l(v, R(0.0175), R(1.0), R(50.0), R(8.0)); }
  __device__ static R bm_NaF(R v) { return l(v, R(7.0), R(0.0), R(65.0), R(20.0)); }
  __device__ static R bh_NaF(R v) { return l(v, R(7.5), R(0.0), R(-3.0), R(-18.0)); }
  __device__ static R bm_NaP(R v) { return l(v, R(25.0), R(1.0), R(58.0), R(8.0)); }
  __device__ static R bm_CaP(R v) { return l(v, R(35.0), R(1.0), R(74.0), R(14.5)); }
  __device__ static R bh_CaP(R v) { return l(v, R(0.0055), R(1.0), R(23.0), R(-8.0)); }
  __device__ static R bm_CaT(R v) { return l(v, R(0.180), R(1.0), R(40.0), R(4.0)); }
  __device__ static R bh_CaT(R v) { return l(v, R(0.190), R(1.0), R(50.0), R(-10.0)); }
  __device__ static R bm_KA(R v) { return l(v, R(0.490), R(1.0), R(30.0), R(4.0)); }
  __device__ static R bh_KA(R v) { return l(v, R(1.30), R(1.0), R(13.0), R(-10.0)); }
  __device__ static R bm_KC(R v) { return l(v, R(0.110), R(0.0), R(-35.0), R(14.9)); }
  __device__ static R bm_K2(R v) { return l(v, R(0.075), R(0.0), R(25.0), R(6.0)); }

  // alpha/beta gate advanced by the trapezoid rule at midpoint voltage v
#define GB_AB(K, A, B)                                                                  \
  {                                                                                      \
    R a_ = A(v), b_ = B(v);                                                              \
    R inf_ = a_ / (a_ + b_), tau_ = R(1.0) / (a_ + b_);                                  \
    s.x(K) = trap(dt, inf_, tau_, s.x(K));                                               \
  }

  // pkj_update_ion_RKC (pkj_ion.cu:304-358); returns nothing, updates state
  __device__ static void ion(const Slots<R> &s, double &v_elem, double &ca, double &rev,
                             double shell, bool rev_fixed, double vnew, double DT) {
    const double v_old = v_elem;
    const double v_val = 0.5 * (vnew + v_old);
    double Ca_val = ca;
    double I = 1e-3 * (v_old - rev) *
               ((double)s.g(PK_g_CaP) * (double)s.x(PK_m_CaP) * (double)s.x(PK_h_CaP) +
                (double)s.g(PK_g_CaT) * (double)s.x(PK_m_CaT) * (double)s.x(PK_h_CaT));
    if (I > 0.0) I = 0.0;
    else I = -I / (2.0 * F_PKJ * shell);
    double k1 = DT * (I - B_Ca1_PKJ * (Ca_val - Ca1_0_PKJ));
    double k2 = DT * (I - B_Ca1_PKJ * (Ca_val + k1 / 2.0 - Ca1_0_PKJ));
    double k3 = DT * (I - B_Ca1_PKJ * (Ca_val + k2 / 2.0 - Ca1_0_PKJ));
    double k4 = DT * (I - B_Ca1_PKJ * (Ca_val + k3 - Ca1_0_PKJ));
    k1 = Ca_val + (k1 + k2 * 2.0 + k3 * 2.0 + k4) / 6.0;
    ca = k1;
    Ca_val = 0.5 * (Ca_val + k1);
    if (rev_fixed) rev = 12.5 * cm_log(Ca1OUT_PKJ / Ca1_0_PKJ);
    else rev = 13.361624877 * cm_log(Ca1OUT_PKJ / Ca_val);
    Ca_val = floor((Ca_val * 1000 - 0.04) / 0.099986667) * 0.099986667 + 0.04;
    const R v = (R)v_val, dt = (R)DT;
    GB_AB(PK_m_NaF, am_NaF, bm_NaF);
    GB_AB(PK_h_NaF, ah_NaF, bh_NaF);
    GB_AB(PK_m_NaP, am_NaP, bm_NaP);
    GB_AB(PK_m_CaP, am_CaP, bm_CaP);
    GB_AB(PK_h_CaP, ah_CaP, bh_CaP);
    GB_AB(PK_m_CaT, am_CaT, bm_CaT);
    GB_AB(PK_h_CaT, ah_CaT, bh_CaT);
    {
      R e = mexp((v + R(82.0)) / R(7.0));
      s.x(PK_m_Kh1) = trap(dt, R(0.8) / (R(1.0) + e), R(7.6), s.x(PK_m_Kh1));
      s.x(PK_m_Kh2) = trap(dt, R(0.2) / (R(1.0) + e), R(36.8), s.x(PK_m_Kh2));
    }
    {
      R a, b;
      if (mabs(v + R(12.0)) > R(1e-6)) a = R(-0.0235) * (v + R(12.0)) / (mexp(-(v + R(12.0)) / R(12.0)) - R(1.0));
      else a = R(0.0235) * R(12.0);
      b = R(5.0) * mexp(-(v + R(147.0)) / R(30.0));
      R tau = R(1.0) / (a + b);
      if (mabs(v - R(8.0)) > R(1e-6)) a = R(-0.0235) * (v - R(8.0)) / (mexp(-(v - R(8.0)) / R(12.0)) - R(1.0));
      else a = R(0.0235) * R(12.0);
      b = R(5.0) * mexp(-(v + R(127.0)) / R(30.0));
      R inf = a / (a + b);
      s.x(PK_m_Kdr) = trap(dt, inf, tau, s.x(PK_m_Kdr));
    }
    s.x(PK_h_Kdr) = trap(dt, R(1.0) / (R(1.0) + mexp((v + R(25.0)) / R(4.0))),
                         (v_val < -25.0) ? R(1200.0) : R(10.0), s.x(PK_h_Kdr));
    s.x(PK_m_KM) = trap(dt, R(1.0) / (R(1.0) + mexp(-(v + R(35.0)) / R(10.0))),
                        R(200.0) / (R(3.3) * (mexp((v + R(35.0)) / R(20.0))) + mexp(-(v + R(35.0)) / R(20.0))),
                        s.x(PK_m_KM));
    GB_AB(PK_m_KA, am_KA, bm_KA);
    GB_AB(PK_h_KA, ah_KA, bh_KA);
    {
      R b_ = bm_KC(v);
      s.x(PK_m_KC) = trap(dt, R(7.5) / (R(7.5) + b_), R(1.0) / (R(7.5) + b_), s.x(PK_m_KC));
    }
    const R caq = (R)Ca_val;
    s.x(PK_z_KC) = trap(dt, R(1.0) / (R(1.0) + R(4.00) / caq), R(10.0), s.x(PK_z_KC));
    {
      R b_ = bm_K2(v);
      s.x(PK_m_K2) = trap(dt, R(25.0) / (R(25.0) + b_), R(1.0) / (R(25.0) + b_), s.x(PK_m_K2));
    }
    s.x(PK_z_K2) = trap(dt, R(1.0) / (R(1.0) + R(0.20) / caq), R(10.0), s.x(PK_z_K2));
    v_elem = vnew;
  }

  // pkj_update_matrix (solve_rkc.cu:370-398)
  __device__ static R b(const Slots<R> &s, double vy, double iext, double rev) {
    const R lv = (R)vy, vca = (R)rev;
    return (-(R)iext + s.g(PK_g_leak) * (lv - R(V_LEAK_PKJ)) +
            s.g(PK_g_NaF) * s.x(PK_m_NaF) * s.x(PK_m_NaF) * s.x(PK_m_NaF) * s.x(PK_h_NaF) * (lv - R(V_Na_PKJ)) +
            s.g(PK_g_NaP) * s.x(PK_m_NaP) * s.x(PK_m_NaP) * s.x(PK_m_NaP) * (lv - R(V_Na_PKJ)) +
            s.g(PK_g_CaP) * s.x(PK_m_CaP) * s.x(PK_h_CaP) * (lv - vca) +
            s.g(PK_g_CaT) * s.x(PK_m_CaT) * s.x(PK_h_CaT) * (lv - vca) +
            s.g(PK_g_Kh) * s.x(PK_m_Kh1) * (lv - R(V_KH_PKJ)) +
            s.g(PK_g_Kh) * s.x(PK_m_Kh2) * (lv - R(V_KH_PKJ)) +
            s.g(PK_g_Kdr) * s.x(PK_m_Kdr) * s.x(PK_m_Kdr) * s.x(PK_h_Kdr) * (lv - R(V_K_PKJ)) +
            s.g(PK_g_KM) * s.x(PK_m_KM) * (lv - R(V_K_PKJ)) +
            s.g(PK_g_KA) * s.x(PK_m_KA) * s.x(PK_m_KA) * s.x(PK_m_KA) * s.x(PK_m_KA) * s.x(PK_h_KA) * (lv - R(V_K_PKJ)) +
            s.g(PK_g_KC) * s.x(PK_m_KC) * s.x(PK_z_KC) * s.x(PK_z_KC) * (lv - R(V_K_PKJ)) +
            s.g(PK_g_K2) * s.x(PK_m_K2) * s.x(PK_z_K2) * s.x(PK_z_K2) * (lv - R(V_K_PKJ)));
  }
};

// ---------------------------------------------------------- inferior olive
template <typename R> struct Io {
  __device__ static R ar(R v) { return (R(1.7)) / (R(1.0) + mexp((-(v - R(5.0))) / R(13.9))); }
  __device__ static R as(R x) { return mmin(R(0.00002) * x, R(0.01)); }
  // 0.13 (v + 25) / (1 - exp(-(v + 25) / 10)) and 0.02 (v + 8.5) / (exp((v + 8.5) / 5) - 1)
  __device__ static R ax(R v) { return hh_xr(R(0.13), v + R(25.0), R(10.0)); }
  __device__ static R br(R v) { return -hh_xr(R(0.02), v + R(8.5), R(-5.0)); }
  __device__ static R bx(R v) { return R(1.69) * mexp(R(-0.0125) * (v + R(35.0))); }
  __device__ static R n_tau(R v) { return R(47.0) * mexp((-(-v - R(50.0))) / R(900.0)) + R(5.0); }

  // io_update_ion_RKC (io_ion.cu:91-126)
  __device__ static void ion(const Slots<R> &s, double &v_elem, double &ca, int comp_type,
                             double vnew, double DT) {
    const double v_old = v_elem;
    const double v_val = 0.5 * (vnew + v_old);
    double Ca_val = ca;
    const double rr = (double)s.x(IO_r);
    double I = (double)s.g(IO_g_CaH) * rr * rr * (v_old - V_Ca_IO);
    double k1 = DT * (-I * CA_PH_IO - BETA_CA_IO * (Ca_val));
    double k2 = DT * (-I * CA_PH_IO - BETA_CA_IO * (Ca_val + k1 / 2.0));
    double k3 = DT * (-I * CA_PH_IO - BETA_CA_IO * (Ca_val + k2 / 2.0));
    double k4 = DT * (-I * CA_PH_IO - BETA_CA_IO * (Ca_val + k3));
    ca += (k1 + k2 * 2.0 + k3 * 2.0 + k4) / 6.0;
    Ca_val = (Ca_val + ca) / 2.0;
    const R v = (R)v_val, dt = (R)DT, c = (R)Ca_val;
    s.x(IO_k) = trap(dt, R(1.0) / (R(1.0) + mexp((-v - R(61.0)) / R(4.2))), R(1.0), s.x(IO_k));
    s.x(IO_l) = trap(dt, R(1.0) / (R(1.0) + mexp((v + R(85.5)) / (R(8.5)))),
                     ((R(20.0) * mexp((v + R(160.0)) / R(30.0))) / (R(1.0) + mexp((v + R(84.0)) / R(7.3)))) + R(35.0),
                     s.x(IO_l));
    const R ntau = n_tau(v);
    s.x(IO_n) = trap(dt, R(1.0) / (R(1.0) + mexp((-v - R(3.0)) / (R(10.0)))), ntau, s.x(IO_n));
    s.x(IO_p) = trap(dt, R(1.0) / (R(1.0) + mexp((-v - R(51.0)) / (R(-12.0)))), ntau, s.x(IO_p));
    {
      R a = ax(v), b = bx(v);
      s.x(IO_x) = trap(dt, a / (a + b), R(1.0) / (a + b), s.x(IO_x));
    }
    {
      R a = ar(v), b = br(v);
      s.x(IO_r) = trap(dt, a / (a + b), R(5.0) / (a + b), s.x(IO_r));
    }
    s.x(IO_q) = trap(dt, R(1.0) / (R(1.0) + mexp((v + R(80.0)) / R(4.0))),
                     R(1.0) / (mexp(R(-0.086) * v - R(14.6)) + mexp(R(0.07) * v - R(1.87))), s.x(IO_q));
    {
      R a = as(c);
      s.x(IO_s) = trap(dt, a / (a + R(0.015)), R(1.0) / (a + R(0.015)), s.x(IO_s));
    }
    s.x(IO_m) = R(1.0) / (R(1.0) + mexp((-v - R(30.0)) / (R(5.5))));
    {
      R hi = R(1.0), ht = R(1.0);
      if (comp_type == 1) {
        hi = R(1.0) / (R(1.0) + mexp((-v - R(70.0)) / (R(-5.8))));
        ht = R(3.0) * mexp((-v - R(40.0)) / R(33.0));
      }
      if (comp_type == 2) {
        hi = R(1.0) / (R(1.0) + mexp((-v - R(60.0)) / (R(-5.8))));
        ht = R(1.5) * mexp((-v - R(40.0)) / R(33.0));
      }
      s.x(IO_h) = trap(dt, hi, ht, s.x(IO_h));
    }
    v_elem = vnew;
  }

  // io_update_matrix (solve_rkc.cu:413-435)
  __device__ static R b(const Slots<R> &s, double vy, double iext) {
    const R lv = (R)vy;
    return (-(R)iext + s.g(IO_g_leak) * (lv - R(V_LEAK_IO)) +
            s.g(IO_g_CaL) * (lv - R(V_Ca_IO)) * s.x(IO_k) * s.x(IO_k) * s.x(IO_k) * s.x(IO_l) +
            s.g(IO_g_Na) * (lv - R(V_Na_IO)) * s.x(IO_m) * s.x(IO_m) * s.x(IO_m) * s.x(IO_h) +
            s.g(IO_g_Kdr) * (lv - R(V_K_IO)) * s.x(IO_n) * s.x(IO_p) +
            s.g(IO_g_K) * (lv - R(V_K_IO)) * s.x(IO_x) * s.x(IO_x) * s.x(IO_x) * s.x(IO_x) +
            s.g(IO_g_CaH) * (lv - R(V_Ca_IO)) * s.x(IO_r) * s.x(IO_r) +
            s.g(IO_g_KCa) * (lv - R(V_K_IO)) * s.x(IO_s) +
            s.g(IO_g_H) * (lv - R(V_H_IO)) * s.x(IO_q));
  }
};

// IO gap-junction current of one directed edge (gap.cu:141-160); FP64
__device__ __forceinline__ double io_gap_current(double g, double diff) {
  return g * (0.8 * cm_exp(-0.01 * diff * diff) + 0.2) * (diff);
}

// ------------------------------------------------------------------ granule
template <typename R> struct Gr {
  __device__ static R a_nKV(R v) {
    return (mabs(v + R(25.0)) > R(1.0e-6)) ? R(-0.017) * ((v + R(25.0)) / (mexp(-(v + R(25.0)) / R(10.0)) - R(1.0)))
                                            : R(-0.17) * (R(1.0) + (v + R(25.0)) / R(20.0));
  }
  __device__ static R b_nKV(R v) { return R(0.2223) * mexp(-(v + R(35.0)) / R(80.0)); }

  // gr_update_ion_RKC_exp_imp (gr_ion.cu:461-480): Ca is never advanced
  __device__ static void ion(const Slots<R> &s, double &v_elem, double ca, double vnew, double DT) {
    const double v_val = (v_elem + vnew) / 2.0;
    const R v = (R)v_val, dt = (R)DT, c = (R)ca;
    {
      R a = a_nKV(v), b = b_nKV(v);
      s.x(GR_n_KV) = trap(dt, a / (a + b), R(1.0) / (a + b), s.x(GR_n_KV));
    }
    {
      R a = R(0.771) / (R(1.0) + mexp(-(v + R(9.17203)) / R(23.32708)));
      R b = R(0.1567) / mexp((v + R(18.27914)) / R(19.47175));
      s.x(GR_a_KA) = trap(dt, R(1.0) / (R(1.0) + mexp(-(v + R(38.0)) / R(17.0))), (R(1.0) / (a + b)), s.x(GR_a_KA));
    }
    {
      R a = R(0.0348) / (R(1.0) + mexp((v + R(111.33208)) / R(12.8433)));
      R b = R(0.0327) / (R(1.0) + mexp(-(v + R(49.9537)) / R(8.90123)));
      s.x(GR_b_KA) = trap(dt, R(1.0) / (R(1.0) + mexp((v + R(78.8)) / R(8.4))), (R(1.0) / (a + b)), s.x(GR_b_KA));
    }
    {
      R a = R(0.2302) * mexp(-(v + R(83.94)) / R(24.3902));
      R b = R(0.2943) * mexp((v + R(83.94)) / R(35.714));
      s.x(GR_ir_KIR) = trap(dt, a / (a + b), R(1.0) / (a + b), s.x(GR_ir_KIR));
    }
    {
      R a = R(0.0046) * mexp((v + R(30.0)) / R(40.0));
      R b = R(0.0046) * mexp(-(v + R(30.0)) / R(20.0));
      s.x(GR_s_KM) = trap(dt, R(1.0) / (R(1.0) + mexp(-(v + R(35.0)) / R(6.0))), (R(1.0) / (a + b)), s.x(GR_s_KM));
    }
    {
      R a = R(1.4433) / (R(1.0) + (R(1.5e-3) * mexp(-v / R(11.765))) / c);
      R b = R(0.8660) / (R(1.0) + c / (R(1.5e-4) * mexp(-v / R(11.765))));
      s.x(GR_c_KCa) = trap(dt, a / (a + b), (R(1.0) / (a + b)), s.x(GR_c_KCa));
    }
    v_elem = vnew;
  }

  // gr_update_matrix (solve_rkc.cu:227-250)
  __device__ static R b(const Slots<R> &s, double vy, double iext) {
    const R lv = (R)vy;
    return (+s.g(GR_g_leak1) * (lv - R(V_LEAK1_GR)) + s.g(GR_g_leak2) * (lv - R(V_LEAK2_GR)) +
            s.g(GR_g_leak3) * (lv - R(V_LEAK3_GR)) - (R)iext +
            +s.g(GR_g_Na) * (lv - R(V_Na_GR)) * s.x(GR_o_Na) +
            s.g(GR_g_Ca) * (lv - R(V_Ca_GR)) * s.x(GR_ch_Ca) * s.x(GR_ch_Ca) * s.x(GR_ci_Ca) +
            s.g(GR_g_KV) * (lv - R(V_K_GR)) * s.x(GR_n_KV) * s.x(GR_n_KV) * s.x(GR_n_KV) * s.x(GR_n_KV) +
            s.g(GR_g_KIR) * (lv - R(V_K_GR)) * s.x(GR_ir_KIR) +
            s.g(GR_g_KA) * (lv - R(V_K_GR)) * s.x(GR_a_KA) * s.x(GR_a_KA) * s.x(GR_a_KA) * s.x(GR_b_KA) +
            s.g(GR_g_KCa) * (lv - R(V_K_GR)) * s.x(GR_c_KCa) +
            s.g(GR_g_KM) * (lv - R(V_K_GR)) * s.x(GR_s_KM));
  }
};

// Partial-pivoting Gaussian elimination on a small dense system, in the
// reference's elimination order (gr_ion.cu:141-190, go_ion.cu:152-200).
// Returns false on a "pivot error" (state left unchanged, as the reference).
template <typename R, int N>
__device__ bool small_solve(R (&A)[N][N], R (&b)[N]) {
#pragma unroll 1
  for (int i = 0; i < N - 1; i++) {
    int piv = i;
    R pmax = mabs(A[i][i]);
    for (int j = i + 1; j < N; j++)
      if (mabs(A[j][i]) > pmax) { piv = j; pmax = mabs(A[j][i]); }
    if (mabs(pmax) < R(1.0e-12)) return false;
    if (piv != i) {
      for (int j = i; j < N; j++) { R t = A[i][j]; A[i][j] = A[piv][j]; A[piv][j] = t; }
      R t = b[i]; b[i] = b[piv]; b[piv] = t;
    }
    for (int j = i + 1; j < N; j++) {
      // A row whose entry in the pivot column is exactly zero has multiplier
      // zero and would be left unchanged (x - y * 0 = x): skip it.  The
      // kinetic matrices are banded, so this removes most of the work while
      // producing the same values as the dense elimination.
      if (A[j][i] == R(0.0)) continue;
      R w = A[j][i] / A[i][i];
      A[j][i] = R(0.0);
      for (int k = i + 1; k < N; k++) A[j][k] = A[j][k] - A[i][k] * w;
      b[j] = b[j] - b[i] * w;
    }
  }
#pragma unroll 1
  for (int i = N - 1; i >= 0; i--) {
    for (int j = i + 1; j < N; j++) b[i] = b[i] - A[i][j] * b[j];
    b[i] = b[i] / A[i][i];
  }
  return true;
}

// Register-resident elimination for the channels' Crank-Nicolson systems.
//
// Both kinetic matrices (GR Na, 12 states; GoC KAHP, 6 states) are
// -(Q + (2/DT) I), Q a rate generator (non-negative off-diagonals, each column
// summing to zero): every column's diagonal exceeds the sum of its
// off-diagonal magnitudes by 2/DT >= 16.  Gaussian elimination preserves
// strict column diagonal dominance, so the partial pivoting of the reference
// (gr_ion.cu:141-190, go_ion.cu:152-200) always keeps the diagonal; rounding
// (relative 1e-7) cannot close a margin that large.  dd_solve therefore runs
// the same elimination without row swaps, fully unrolled over the compile-time
// fill-in pattern of the matrix so it stays in registers.  It still checks
// every pivot and returns DD_PIVOT if a swap would have been taken (the
// caller then reruns the dense pivoting solver): results are the dense
// solver's in every case.  Entries outside the pattern are exactly zero; the
// dense solver's updates with them leave every value unchanged (up to the
// sign of a zero), so they are skipped.
enum { DD_OK = 0, DD_SINGULAR = 1, DD_PIVOT = 2 };

template <int N>
struct Fill {
  uint32_t r[N];  // bit k of r[i]: entry (i, k) may be nonzero
};

template <int N>
constexpr Fill<N> fill_in(const uint32_t (&rows)[N]) {
  Fill<N> f{};
  for (int i = 0; i < N; i++) f.r[i] = rows[i] | (1u << i);
  for (int i = 0; i < N - 1; i++)
    for (int j = i + 1; j < N; j++)
      if ((f.r[j] >> i) & 1u) f.r[j] |= f.r[i] & ~((2u << i) - 1u);
  return f;
}

template <int N>
constexpr Fill<N> as_fill(const uint32_t (&rows)[N]) {
  Fill<N> f{};
  for (int i = 0; i < N; i++) f.r[i] = rows[i];
  return f;
}

#define GB_ROW(...) gb_bits({__VA_ARGS__})
template <int K>
constexpr uint32_t gb_bits(const int (&cols)[K]) {
  uint32_t m = 0;
  for (int k = 0; k < K; k++) m |= 1u << cols[k];
  return m;
}

// nonzero pattern of the GR Na matrix (gr_na_fill)
struct NaPattern {
  static constexpr int N = 12;
  static constexpr uint32_t rows[12] = {
      GB_ROW(0, 1, 5),      GB_ROW(0, 1, 2, 6),   GB_ROW(1, 2, 3, 7),   GB_ROW(2, 3, 4, 8),
      GB_ROW(3, 4, 9, 11),  GB_ROW(0, 5, 6),      GB_ROW(1, 5, 6, 7),   GB_ROW(2, 6, 7, 8),
      GB_ROW(3, 7, 8, 9),   GB_ROW(4, 8, 9, 10),  GB_ROW(9, 10, 11),    GB_ROW(4, 10, 11)};
  static constexpr Fill<12> fill = fill_in<12>(rows);
  static constexpr Fill<12> orig = as_fill<12>(rows);
};

// nonzero pattern of the GoC KAHP matrix (Go::kahp)
struct KahpPattern {
  static constexpr int N = 6;
  static constexpr uint32_t rows[6] = {GB_ROW(0, 1),       GB_ROW(0, 1, 2),    GB_ROW(1, 2, 3, 4),
                                       GB_ROW(2, 3, 5),    GB_ROW(2, 4),       GB_ROW(3, 5)};
  static constexpr Fill<6> fill = fill_in<6>(rows);
  static constexpr Fill<6> orig = as_fill<6>(rows);
};
#undef GB_ROW

template <typename R, class PAT>
__device__ __forceinline__ int dd_solve(R (&A)[PAT::N][PAT::N], R (&b)[PAT::N]) {
  constexpr int N = PAT::N;
  constexpr Fill<N> F = PAT::fill;
#pragma unroll
  for (int i = 0; i < N - 1; i++) {
    const R d = mabs(A[i][i]);
#pragma unroll
    for (int j = i + 1; j < N; j++)
      if ((F.r[j] >> i) & 1u)
        if (mabs(A[j][i]) > d) return DD_PIVOT;
    if (d < R(1.0e-12)) return DD_SINGULAR;
#pragma unroll
    for (int j = i + 1; j < N; j++) {
      if (!((F.r[j] >> i) & 1u)) continue;
      if (A[j][i] == R(0.0)) continue;
      const R w = A[j][i] / A[i][i];
      A[j][i] = R(0.0);
#pragma unroll
      for (int k = i + 1; k < N; k++)
        if ((F.r[i] >> k) & 1u) A[j][k] = A[j][k] - A[i][k] * w;
      b[j] = b[j] - b[i] * w;
    }
  }
#pragma unroll
  for (int i = N - 1; i >= 0; i--) {
#pragma unroll
    for (int j = i + 1; j < N; j++)
      if ((F.r[i] >> j) & 1u) b[i] = b[i] - A[i][j] * b[j];
    b[i] = b[i] / A[i][i];
  }
  return DD_OK;
}

// rhs = -M x over the pattern (the dense product's zero terms change nothing)
template <typename R, class PAT>
__device__ __forceinline__ void dd_neg_matvec(const R (&M)[PAT::N][PAT::N], const R (&x)[PAT::N], R (&y)[PAT::N]) {
  constexpr int N = PAT::N;
  constexpr Fill<N> O = PAT::orig;
#pragma unroll
  for (int i = 0; i < N; i++) {
    R acc = R(0.0);
#pragma unroll
    for (int j = 0; j < N; j++)
      if ((O.r[i] >> j) & 1u) acc -= x[j] * M[i][j];
    y[i] = acc;
  }
}

// GR 12-state Na channel, Crank-Nicolson step (gr_ion.cu:45-207).  The
// per-compartment-type constants a = (Oon/Con)^0.25, b = (Ooff/Coff)^0.25,
// a^4, b^4 come precomputed from the host (NaPar).
template <typename R>
__device__ void gr_na_fill(R (&M)[12][12], const NaPar &p, R alpha, R beta, R tdt, bool implicit_half) {
  const R n1 = (R)p.n1, n2 = (R)p.n2, n3 = (R)p.n3, n4 = (R)p.n4;
  const R Con = (R)p.Con, Coff = (R)p.Coff, Oon = (R)p.Oon, Ooff = (R)p.Ooff;
  const R a = (R)p.a, b = (R)p.b, a4 = (R)p.a4, b4 = (R)p.b4;
#pragma unroll
  for (int i = 0; i < 12; i++)
#pragma unroll
    for (int j = 0; j < 12; j++) M[i][j] = R(0.0);
  if (!implicit_half) {
    M[0][0] = -(n1 * alpha + Con - tdt);
    M[1][1] = -(n4 * beta + n2 * alpha + Con * a - tdt);
    M[2][2] = -(n3 * beta + n3 * alpha + Con * a * a - tdt);
    M[3][3] = -(n2 * beta + n4 * alpha + Con * a * a * a - tdt);
    M[4][4] = -(n1 * beta + R(259.8) + Con * a4 - tdt);
    M[5][5] = -(Coff + n1 * alpha * a - tdt);
    M[6][6] = -(Coff * b + n4 * beta * b + n2 * alpha * a - tdt);
    M[7][7] = -(Coff * b * b + n3 * beta * b + n3 * alpha * a - tdt);
    M[8][8] = -(Coff * b * b * b + n2 * beta * b + n4 * alpha * a - tdt);
    M[9][9] = -(Coff * b4 + n1 * beta * b + R(259.8) - tdt);
    M[10][10] = -(Ooff + R(69.3) - tdt);
    M[11][11] = -(R(69.3) + Oon - tdt);
  } else {
    M[0][0] = -(n1 * alpha + Con + tdt);
    M[1][1] = -(n4 * beta + n2 * alpha + Con * a + tdt);
    M[2][2] = -(n3 * beta + n3 * alpha + Con * a * a + tdt);
    M[3][3] = -(n2 * beta + n4 * alpha + Con * a * a * a + tdt);
    M[4][4] = -(n1 * beta + R(259.8) + Con * a4 + tdt);
    M[5][5] = -(Coff + n1 * alpha * a + tdt);
    M[6][6] = -(Coff * b + n4 * beta * b + n2 * alpha * a + tdt);
    M[7][7] = -(Coff * b * b + n3 * beta * b + n3 * alpha * a + tdt);
    M[8][8] = -(Coff * b * b * b + n2 * beta * b + n4 * alpha * a + tdt);
    M[9][9] = -(Coff * b4 + n1 * beta * b + R(259.8) + tdt);
    M[10][10] = -(Ooff + R(69.3) + tdt);
    M[11][11] = -(R(69.3) + Oon + tdt);
  }
  M[0][1] = n4 * beta; M[0][5] = Coff;
  M[1][0] = n1 * alpha; M[1][2] = n3 * beta; M[1][6] = Coff * b;
  M[2][1] = n2 * alpha; M[2][3] = n2 * beta; M[2][7] = Coff * b * b;
  M[3][2] = n3 * alpha; M[3][4] = n1 * beta; M[3][8] = Coff * b * b * b;
  M[4][3] = n4 * alpha; M[4][9] = Coff * b4; M[4][11] = R(69.3);
  M[5][0] = Con; M[5][6] = n4 * beta * b;
  M[6][1] = Con * a; M[6][5] = n1 * alpha * a; M[6][7] = n3 * beta * b;
  M[7][2] = Con * a * a; M[7][6] = n2 * alpha * a; M[7][8] = n2 * beta * b;
  M[8][3] = Con * a * a * a; M[8][7] = n3 * alpha * a; M[8][9] = n1 * beta * b;
  M[9][4] = Con * a4; M[9][8] = n4 * alpha * a; M[9][10] = R(69.3);
  M[10][9] = R(259.8); M[10][11] = Oon;
  M[11][4] = R(259.8); M[11][10] = Ooff;
}

template <typename R>
__device__ void gr_na(const Slots<R> &s, const NaPar &p, double v_new, double v_old, double DT) {
  // state order {c1..c5, i1..i6, o} (gr_ion.cu:104-105)
  const int slot[12] = {GR_c1, GR_c2, GR_c3, GR_c4, GR_c5, GR_i1, GR_i2, GR_i3, GR_i4, GR_i5, GR_i6, GR_o_Na};
  const R vs = (R)p.vshift, tdt = R(2.0) / (R)DT;
  R M[12][12], vc[12], vcb[12];
  const R vo = (R)v_old, vn = (R)v_new;
  const R alpha0 = (R)p.Aa * mexp((vo - vs) / R(10.0));
  const R beta0 = (R)p.Ab * mexp(-(vo - vs) / R(10.0));
  gr_na_fill(M, p, alpha0, beta0, tdt, false);
#pragma unroll
  for (int k = 0; k < 12; k++) vc[k] = s.x(slot[k]);
  dd_neg_matvec<R, NaPattern>(M, vc, vcb);
  const R alpha = (R)p.Aa * mexp((vn - vs) / R(10.0));
  const R beta = (R)p.Ab * mexp(-(vn - vs) / R(10.0));
  gr_na_fill(M, p, alpha, beta, tdt, true);
  const int rc = dd_solve<R, NaPattern>(M, vcb);
  if (rc == DD_SINGULAR) return;
  if (rc == DD_PIVOT) {
    // never reached for these matrices (see dd_solve); the dense pivoting
    // elimination on a fresh copy keeps the result exact regardless
    R A[12][12], rb[12];
    gr_na_fill(A, p, alpha0, beta0, tdt, false);
    dd_neg_matvec<R, NaPattern>(A, vc, rb);
    gr_na_fill(A, p, alpha, beta, tdt, true);
    if (!small_solve<R, 12>(A, rb)) return;
#pragma unroll
    for (int k = 0; k < 12; k++) vcb[k] = rb[k];
  }
#pragma unroll
  for (int k = 0; k < 12; k++) s.x(slot[k]) = vcb[k];
}

// ------------------------------------------------------------------- Golgi
template <typename R> struct Go {
  // go_update_ion_RKC_exp_imp (go_ion.cu:379-437)
  __device__ static void ion(const Slots<R> &s, double &v_elem, double &ca, double &ca2, double &rev,
                             double area, double vnew, double DT) {
    const double v_old = v_elem;
    const double v_val = (v_old + vnew) / 2.0;
    double Ca_val = ca;
    const double Ca2_val = ca2;
    const double ch = (double)s.x(GO_ch), ci = (double)s.x(GO_ci);
    const double cl = (double)s.x(GO_cl), cmv = (double)s.x(GO_cm);
    double I1 = 1e-3 * (double)s.g(GO_g_CaHVA) / area * ch * ch * ci * (v_old - V_Ca_GO);
    double I2 = 1e-3 * (double)s.g(GO_g_CaLVA) / area * cl * cl * cmv * (v_old - (rev));
    double k1 = DT * (-I1 / (2.0 * F_GO * SHELL1_D_GO) - B_Ca1_GO * (Ca_val - Ca1_0_GO));
    double k2 = DT * (-I1 / (2.0 * F_GO * SHELL1_D_GO) - B_Ca1_GO * (Ca_val + k1 / 2.0 - Ca1_0_GO));
    double k3 = DT * (-I1 / (2.0 * F_GO * SHELL1_D_GO) - B_Ca1_GO * (Ca_val + k2 / 2.0 - Ca1_0_GO));
    double k4 = DT * (-I1 / (2.0 * F_GO * SHELL1_D_GO) - B_Ca1_GO * (Ca_val + k3 - Ca1_0_GO));
    ca += (k1 + k2 * 2.0 + k3 * 2.0 + k4) / 6.0;
    k1 = DT * (-I2 / (2.0 * F_GO * SHELL1_D_GO) - B_Ca1_GO * (Ca2_val - Ca1_0_GO));
    k2 = DT * (-I2 / (2.0 * F_GO * SHELL1_D_GO) - B_Ca1_GO * (Ca2_val + k1 / 2.0 - Ca1_0_GO));
    k3 = DT * (-I2 / (2.0 * F_GO * SHELL1_D_GO) - B_Ca1_GO * (Ca2_val + k2 / 2.0 - Ca1_0_GO));
    k4 = DT * (-I2 / (2.0 * F_GO * SHELL1_D_GO) - B_Ca1_GO * (Ca2_val + k3 - Ca1_0_GO));
    ca2 += (k1 + k2 * 2.0 + k3 * 2.0 + k4) / 6.0;
    rev = (1e3) * (8.313424 * (23.0 + 273.15)) / (2 * F_GO) * cm_log(Ca1OUT_GO / ca2);
    Ca_val = (Ca_val + ca) / 2.0;
    const R v = (R)v_val, dt = (R)DT, c = (R)Ca_val;
    {  // m_NaT
      R a = hh_xr(R(0.417), v + R(25.0), R(10.0));
      R b = R(16.68) * mexp(R(-0.055) * (v + R(50.0)));
      s.x(GO_m_NaT) = trap(dt, a / (a + b), R(1.0) / (a + b), s.x(GO_m_NaT));
    }
    {  // h_NaT
      R a = R(0.292) * mexp(R(-0.3) * (v + R(50.0)));
      R b = R(4.17) / (R(1) + mexp(-(v + R(17.0)) / R(5.0)));
      s.x(GO_h_NaT) = trap(dt, a / (a + b), R(1.0) / (a + b), s.x(GO_h_NaT));
    }
    {  // r_NaR
      // (1.11 - 68.5 (v - 4.48) / (exp(-(v - 4.48) / 6.8) - 1)) 1e-4
      R a = ((R(1.11) + hh_xr(R(68.5), v - R(4.48), R(6.8))) * R(1.0e-4));
      R x = (v + R(44.0)) / R(0.11);
      if (x > R(200.0)) x = R(200.0);
      R b;
      if (sizeof(R) == 4 && mabs(x) < R(1e-3))  // the same guard: 21.7 (v + 44) / (e^x - 1) -> 21.7 * 0.11
        b = (R(66.0) + R(21.7) * R(0.11) * (R(1) - x * (R(0.5) - x * R(1.0 / 12.0)))) * R(1.0e-3);
      else
        b = ((R(66.0) + R(21.7) * (v + R(44)) / (mexp(x) - R(1.0))) * R(1.0e-3));
      s.x(GO_r_NaR) = trap(dt, a / (a + b), R(1.0) / (a + b), s.x(GO_r_NaR));
    }
    {  // s_NaR
      R a = (R(0.443) * mexp(-(v + R(80.0)) / R(62.5)));
      R b = (R(0.014) * mexp((v + R(83.3)) / R(16.1)));
      s.x(GO_s_NaR) = trap(dt, a / (a + b), R(1.0) / (a + b), s.x(GO_s_NaR));
    }
    {  // p_NaP
      R a = hh_xr(R(0.421), v + R(40.0), R(5.0));
      R b = hh_xr(R(-0.287), v + R(40.0), R(-5.0));  // -0.287 (v + 40) / (1 - exp((v + 40) / 5))
      s.x(GO_p_NaP) = trap(dt, (R(1) / (R(1.0) + mexp(-(v + R(43.0)) / R(5.0)))), (R(5.0) / (a + b)), s.x(GO_p_NaP));
    }
    {  // n_KV
      R a = hh_xr(R(0.062), v + R(26.0), R(10.0));
      R b = R(0.78) * mexp(-(v + R(36.0)) / R(80.0));
      s.x(GO_n_KV) = trap(dt, a / (a + b), R(1.0) / (a + b), s.x(GO_n_KV));
    }
    {  // a_KA
      R a = (R(0.62) / (R(1.0) + mexp(-(v + R(9.17)) / R(23.32))));
      R b = (R(0.126) / (mexp((v + R(18.28)) / R(19.47))));
      s.x(GO_a_KA) = trap(dt, (R(1.0) / (R(1.0) + mexp(-(v + R(38.0)) / R(17.0)))), (R(1.0) / (a + b)), s.x(GO_a_KA));
    }
    {  // b_KA
      R a = (R(0.028) / (R(1.0) + mexp((v + R(111.0)) / R(12.84))));
      R b = (R(0.026) / (R(1.0) + mexp(-(v + R(49.95)) / R(8.9))));
      s.x(GO_b_KA) = trap(dt, (R(1.0) / (R(1.0) + mexp((v + R(78.8)) / R(8.4)))), (R(1.0) / (a + b)), s.x(GO_b_KA));
    }
    {  // sl_Kslow
      R a = (R(0.0037) * mexp((v + R(30.0)) / R(40.0)));
      R b = (R(0.0037) * mexp(-(v + R(30.0)) / R(20.0)));
      s.x(GO_sl) = trap(dt, (R(1.0) / (R(1.0) + mexp(-(v + R(35.0)) / R(6.0)))), (R(1.0) / (a + b)), s.x(GO_sl));
    }
    {  // c_KC (Ca-dependent)
      R a = (R(3.2) / (R(1.0) + R(0.0015) * mexp(-(v) / R(11.7)) / c));
      R b = (R(0.46) / (R(1.0) + c / (R(1.5e-4) * mexp(-(v) / R(11.7)))));
      s.x(GO_c_KC) = trap(dt, (a / (a + b)), (R(1.0) / (a + b)), s.x(GO_c_KC));
    }
    {  // ch_CaHVA
      R a = (R(0.0687) * mexp(R(0.063) * (v + R(29.0))));
      R b = (R(0.115) * mexp(R(-0.039) * (v + R(18.66))));
      s.x(GO_ch) = trap(dt, (a / (a + b)), (R(1.0) / (a + b)), s.x(GO_ch));
    }
    {  // ci_CaHVA
      R a = (R(1.8e-3) * mexp(-(v + R(48.0)) / R(18.0)));
      R b = (R(1.8e-3) * mexp((v + R(48.0)) / R(83.0)));
      s.x(GO_ci) = trap(dt, (a / (a + b)), (R(1.0) / (a + b)), s.x(GO_ci));
    }
    s.x(GO_cl) = trap(dt, (R(1.0) / (R(1.0) + mexp(-(v + R(52.0)) / R(7.4)))),
                      ((R(3.0) + R(1.0) / (mexp((v + R(27.0)) / R(10.0)) + mexp(-(v + R(102.0)) / R(15.0)))) / R(0.85)),
                      s.x(GO_cl));
    s.x(GO_cm) = trap(dt, (R(1.0) / (R(1.0) + mexp((v + R(80.0)) / R(5.0)))),
                      ((R(85.0) + R(1.0) / (mexp((v + R(48.0)) / R(4.0)) + mexp(-(v + R(407.0)) / R(50.0)))) / R(0.9)),
                      s.x(GO_cm));
    {  // HCN1 / HCN2 (r_HCN2 ramp decided on the FP64 voltage)
      const R r1 = (R(0.0021) * (v) + R(0.97));
      const R s1 = (R(1.0) / (R(1.0) + mexp((v + R(72.5)) * R(0.11))));
      R r2;
      if (v_val >= -64.70) r2 = R(0.0);
      else if (v_val <= -108.70) r2 = R(1.0);
      else r2 = (R(-0.0227) * (v) - R(1.47));
      const R s2 = (R(1.0) / (R(1.0) + mexp((v + R(81.9)) * R(0.16))));
      s.x(GO_hf1) = trap(dt, (r1 * s1), (mexp((R(0.0137) * v + R(3.37)) * R(2.3))), s.x(GO_hf1));
      s.x(GO_hf2) = trap(dt, (r2 * s2), (mexp((R(0.027) * v + R(5.6)) * R(2.3))), s.x(GO_hf2));
      s.x(GO_hs1) = trap(dt, ((R(1.0) - r1) * s1), (mexp((R(0.0145) * v + R(4.06)) * R(2.3))), s.x(GO_hs1));
      s.x(GO_hs2) = trap(dt, ((R(1.0) - r2) * s2), (mexp((R(0.015) * v + R(5.3)) * R(2.3))), s.x(GO_hs2));
    }
    v_elem = vnew;
  }

  // go_KAHP_update_2order (go_ion.cu:88-213)
  __device__ static void kahp(const Slots<R> &s, double ca_new, double &ca_old, double DT) {
    const R i1 = R(80e-3), i2 = R(80e-3), i3 = R(200e-3), a1 = R(1.0), a2 = R(100e-3), b1 = R(160e-3), b2 = R(1.2);
    R l_ca = (R)ca_old;
    ca_old = ca_new;
    const R l_dt = R(2.0) / (R)DT;
    R d1 = R(200) * l_ca / R(3.0), d2 = R(160) * l_ca / R(3.0), d3 = R(80) * l_ca / R(3.0);
    const int slot[6] = {GO_c1, GO_c2, GO_c3, GO_c4, GO_o1, GO_o2};
    R vc[6], vcb[6];
#pragma unroll
    for (int k = 0; k < 6; k++) vc[k] = s.x(slot[k]);
    R E[6][6] = {{-d1 + l_dt, i1, R(0), R(0), R(0), R(0)},
                 {d1, -d2 - i1 + l_dt, i2, R(0), R(0), R(0)},
                 {R(0), d2, -(d3 + i2 + b1) + l_dt, i3, a1, R(0)},
                 {R(0), R(0), d3, -(i3 + b2) + l_dt, R(0), a2},
                 {R(0), R(0), b1, R(0), -a1 + l_dt, R(0)},
                 {R(0), R(0), R(0), b2, R(0), -a2 + l_dt}};
    dd_neg_matvec<R, KahpPattern>(E, vc, vcb);
    l_ca = (R)ca_new;
    d1 = R(200) * l_ca / R(3.0); d2 = R(160) * l_ca / R(3.0); d3 = R(80) * l_ca / R(3.0);
    R M[6][6] = {{-d1 - l_dt, i1, R(0), R(0), R(0), R(0)},
                 {d1, -d2 - i1 - l_dt, i2, R(0), R(0), R(0)},
                 {R(0), d2, -(d3 + i2 + b1) - l_dt, i3, a1, R(0)},
                 {R(0), R(0), d3, -(i3 + b2) - l_dt, R(0), a2},
                 {R(0), R(0), b1, R(0), -a1 - l_dt, R(0)},
                 {R(0), R(0), R(0), b2, R(0), -a2 - l_dt}};
    const int rc = dd_solve<R, KahpPattern>(M, vcb);
    if (rc == DD_SINGULAR) return;
    if (rc == DD_PIVOT) {
      // never reached (see dd_solve); the dense pivoting solver on a fresh copy
      R A[6][6] = {{-d1 - l_dt, i1, R(0), R(0), R(0), R(0)},
                   {d1, -d2 - i1 - l_dt, i2, R(0), R(0), R(0)},
                   {R(0), d2, -(d3 + i2 + b1) - l_dt, i3, a1, R(0)},
                   {R(0), R(0), d3, -(i3 + b2) - l_dt, R(0), a2},
                   {R(0), R(0), b1, R(0), -a1 - l_dt, R(0)},
                   {R(0), R(0), R(0), b2, R(0), -a2 - l_dt}};
      R rb[6];
      dd_neg_matvec<R, KahpPattern>(E, vc, rb);
      if (!small_solve<R, 6>(A, rb)) return;
#pragma unroll
      for (int k = 0; k < 6; k++) vcb[k] = rb[k];
    }
#pragma unroll
    for (int k = 0; k < 6; k++) s.x(slot[k]) = vcb[k];
  }

  // go_update_matrix (solve_rkc.cu:289-312)
  __device__ static R b(const Slots<R> &s, double vy, double iext, double rev) {
    const R lv = (R)vy;
    return (-(R)iext + s.g(GO_g_leak) * (lv - R(V_LEAK_GO)) +
            s.g(GO_g_NaT) * (lv - R(V_Na_GO)) * s.x(GO_m_NaT) * s.x(GO_m_NaT) * s.x(GO_m_NaT) * s.x(GO_h_NaT) +
            s.g(GO_g_NaR) * (lv - R(V_Na_GO)) * s.x(GO_r_NaR) * s.x(GO_s_NaR) +
            s.g(GO_g_NaP) * (lv - R(V_Na_GO)) * s.x(GO_p_NaP) +
            s.g(GO_g_CaHVA) * (lv - R(V_Ca_GO)) * s.x(GO_ch) * s.x(GO_ch) * s.x(GO_ci) +
            s.g(GO_g_CaLVA) * (lv - (R)rev) * s.x(GO_cl) * s.x(GO_cl) * s.x(GO_cm) +
            s.g(GO_g_KAHP) * (lv - R(V_K_GO)) * (s.x(GO_o1) + s.x(GO_o2)) +
            s.g(GO_g_KV) * (lv - R(V_K_GO)) * s.x(GO_n_KV) * s.x(GO_n_KV) * s.x(GO_n_KV) * s.x(GO_n_KV) +
            s.g(GO_g_KA) * (lv - R(V_K_GO)) * s.x(GO_a_KA) * s.x(GO_a_KA) * s.x(GO_a_KA) * s.x(GO_b_KA) +
            s.g(GO_g_KC) * (lv - R(V_K_GO)) * s.x(GO_c_KC) +
            s.g(GO_g_Kslow) * (lv - R(V_K_GO)) * s.x(GO_sl) +
            s.g(GO_g_HCN1) * (lv - R(V_H_GO)) * (s.x(GO_hf1) + s.x(GO_hs1)) +
            s.g(GO_g_HCN2) * (lv - R(V_H_GO)) * (s.x(GO_hf2) + s.x(GO_hs2)));
  }
};
#undef GB_AB

}  // namespace gbrkc

// Host-side initial state of each cell type: the reference's *_initialize_ion
// (gr_ion.cu:635-672, go_ion.cu:590-634, pkj_ion.cu:360-395,
// io_ion.cu:163-194).  The reference computes these on the host with the C
// library's exp, and so does this file (built with -ffp-contract=off); the
// resulting gates are bit-identical to the oracle's.
#include <math.h>

#include "host_init.h"
#include "model.h"

namespace gbrkc {
namespace {

double ab(double a, double b) { return a / (a + b); }

// Purkinje rate pieces (pkj_ion.cu:4-91)
double pl(double v, double A, double B, double C, double D) { return A / (B + exp((v + C) / D)); }

void pkj_init(double v, double ca, double *x) {
  x[PK_m_NaF] = ab(pl(v, 35.0, 0.0, 5.0, -10.0), pl(v, 7.0, 0.0, 65.0, 20.0));
  x[PK_h_NaF] = ab(pl(v, 0.225, 1.0, 80.0, 10.0), pl(v, 7.5, 0.0, -3.0, -18.0));
  x[PK_m_NaP] = ab(pl(v, 200.0, 1.0, -18.0, -16.0), pl(v, 25.0, 1.0, 58.0, 8.0));
  x[PK_m_CaP] = ab(pl(v, 8.5, 1.0, -8.0, -12.5), pl(v, 35.0, 1.0, 74.0, 14.5));
  x[PK_h_CaP] = ab(pl(v, 0.0015, 1.0, 29.0, 8.0), pl(v, 0.0055, 1.0, 23.0, -8.0));
  x[PK_m_CaT] = ab(pl(v, 2.60, 1.0, 21.0, -8.0), pl(v, 0.180, 1.0, 40.0, 4.0));
  x[PK_h_CaT] = ab(pl(v, 0.0025, 1.0, 40.0, 8.0), pl(v, 0.190, 1.0, 50.0, -10.0));
  x[PK_m_Kh1] = 0.8 / (1.0 + exp((v + 82.0) / 7.0));
  x[PK_m_Kh2] = 0.2 / (1.0 + exp((v + 82.0) / 7.0));
  {
    double a;
    if (fabs(v - 8.0) > 1e-6) a = -0.0235 * (v - 8.0) / (exp(-(v - 8.0) / 12.0) - 1.0);
    else a = 0.0235 * 12.0;
    double b = 5.0 * exp(-(v + 127.0) / 30.0);
    x[PK_m_Kdr] = a / (a + b);
  }
  x[PK_h_Kdr] = 1.0 / (1.0 + exp((v + 25.0) / 4.0));
  x[PK_m_KM] = 1.0 / (1.0 + exp(-(v + 35.0) / 10.0));
  x[PK_m_KA] = ab(pl(v, 1.40, 1.0, 27.0, -12.0), pl(v, 0.490, 1.0, 30.0, 4.0));
  x[PK_h_KA] = ab(pl(v, 0.0175, 1.0, 50.0, 8.0), pl(v, 1.30, 1.0, 13.0, -10.0));
  x[PK_m_KC] = 7.5 / (7.5 + pl(v, 0.110, 0.0, -35.0, 14.9));
  x[PK_z_KC] = 1.0 / (1.0 + 4.00 / ca);
  x[PK_m_K2] = 25.0 / (25.0 + pl(v, 0.075, 0.0, 25.0, 6.0));
  x[PK_z_K2] = 1.0 / (1.0 + 0.20 / ca);
}

// inferior olive (io_ion.cu:5-51)
double io_ar(double v) { return (1.7) / (1.0 + exp((-(v - 5.0)) / 13.9)); }
double io_br(double v) { return (0.02 * (v + 8.5)) / (exp((v + 8.5) / 5.0) - 1.0); }
double io_ax(double v) { return (0.13 * (v + 25.0)) / (1.0 - exp(-(v + 25.0) / 10.0)); }
double io_bx(double v) { return 1.69 * exp(-0.0125 * (v + 35.0)); }

void io_init(double v, int comp_type, double g_CaH, double *ca, double *x) {
  x[IO_k] = 1.0 / (1.0 + exp((-v - 61.0) / 4.2));
  x[IO_l] = 1.0 / (1.0 + exp((v + 85.5) / (8.5)));
  x[IO_n] = 1.0 / (1.0 + exp((-v - 3.0) / (10.0)));
  x[IO_p] = 1.0 / (1.0 + exp((-v - 51.0) / (-12.0)));
  x[IO_x] = io_ax(v) / (io_ax(v) + io_bx(v));
  x[IO_r] = io_ar(v) / (io_ar(v) + io_br(v));
  x[IO_q] = 1.0 / (1.0 + exp((v + 80.0) / 4.0));
  double I = g_CaH * x[IO_r] * x[IO_r] * (v - V_Ca_IO);
  *ca = -I * CA_PH_IO / BETA_CA_IO;
  double as = fmin(0.00002 * *ca, 0.01);
  x[IO_s] = as / (as + 0.015);
  x[IO_m] = 1.0 / (1.0 + exp((-v - 30.0) / (5.5)));
  double h = 1.0;
  if (comp_type == 1) h = 1.0 / (1.0 + exp((-v - 70.0) / (-5.8)));
  if (comp_type == 2) h = 1.0 / (1.0 + exp((-v - 60.0) / (-5.8)));
  x[IO_h] = h;
}

// granule cell (gr_ion.cu:3-43)
void gr_init(double v, double ca, double *x) {
  {
    double a = (fabs(v + 25.0) > 1.0e-6) ? -0.017 * ((v + 25.0) / (exp(-(v + 25.0) / 10.0) - 1.0))
                                         : -0.17 * (1.0 + (v + 25.0) / 20.0);
    double b = 0.2223 * exp(-(v + 35.0) / 80.0);
    x[GR_n_KV] = a / (a + b);
  }
  x[GR_a_KA] = 1.0 / (1.0 + exp(-(v + 38.0) / 17.0));
  x[GR_b_KA] = 1.0 / (1.0 + exp((v + 78.8) / 8.4));
  x[GR_ir_KIR] = ab(0.2302 * exp(-(v + 83.94) / 24.3902), 0.2943 * exp((v + 83.94) / 35.714));
  x[GR_s_KM] = 1.0 / (1.0 + exp(-(v + 35.0) / 6.0));
  {
    double a = 1.4433 / (1.0 + (1.5e-3 * exp(-v / 11.765)) / ca);
    double b = 0.8660 / (1.0 + ca / (1.5e-4 * exp(-v / 11.765)));
    x[GR_c_KCa] = a / (a + b);
  }
  x[GR_ch_Ca] = ab(0.0856 * exp((v + 29.6) / 15.873), 0.1437 * exp(-(v + 18.66) / 25.641));
  x[GR_ci_Ca] = ab(0.0023 * exp(-(v + 48.0) / 18.183), 0.0025 * exp((v + 48.0) / 83.33));
  for (int k = GR_o_Na; k <= GR_i6; k++) x[k] = 0.0;
  x[GR_c1] = 1.0;
}

// Golgi cell (go_ion.cu:3-86)
void go_init(double v, double ca, double *x) {
  x[GO_m_NaT] = ab(0.417 * (v + 25.0) / (1 - exp(-(v + 25.0) / 10.0)), 16.68 * exp(-0.055 * (v + 50.0)));
  x[GO_h_NaT] = ab(0.292 * exp(-0.3 * (v + 50.0)), 4.17 / (1 + exp(-(v + 17.0) / 5.0)));
  {
    double a = ((1.11 - 68.5 * (v - 4.48) / (exp(-(v - 4.48) / 6.8) - 1.0)) * 1.0e-4);
    double xx = (v + 44.0) / 0.11;
    if (xx > 200.0) xx = 200.0;
    double b = ((66.0 + 21.7 * (v + 44) / (exp(xx) - 1.0)) * 1.0e-3);
    x[GO_r_NaR] = a / (a + b);
  }
  x[GO_s_NaR] = ab((0.443 * exp(-(v + 80.0) / 62.5)), (0.014 * exp((v + 83.3) / 16.1)));
  x[GO_p_NaP] = (1 / (1.0 + exp(-(v + 43.0) / 5.0)));
  x[GO_n_KV] = ab(0.062 * (v + 26.0) / (1.0 - exp(-(v + 26.0) / 10.0)), 0.78 * exp(-(v + 36.0) / 80.0));
  x[GO_a_KA] = (1.0 / (1.0 + exp(-(v + 38.0) / 17.0)));
  x[GO_b_KA] = (1.0 / (1.0 + exp((v + 78.8) / 8.4)));
  {
    double a = (3.2 / (1.0 + 0.0015 * exp(-(v) / 11.7) / ca));
    double b = (0.46 / (1.0 + ca / (1.5e-4 * exp(-(v) / 11.7))));
    x[GO_c_KC] = (a / (a + b));
  }
  x[GO_sl] = (1.0 / (1.0 + exp(-(v + 35.0) / 6.0)));
  x[GO_ch] = ab((0.0687 * exp(0.063 * (v + 29.0))), (0.115 * exp(-0.039 * (v + 18.66))));
  x[GO_ci] = ab((1.8e-3 * exp(-(v + 48.0) / 18.0)), (1.8e-3 * exp((v + 48.0) / 83.0)));
  x[GO_cl] = (1.0 / (1.0 + exp(-(v + 52.0) / 7.4)));
  x[GO_cm] = (1.0 / (1.0 + exp((v + 80.0) / 5.0)));
  const double r1 = (0.0021 * (v) + 0.97);
  double r2;
  if (v >= -64.70) r2 = 0.0;
  else if (v <= -108.70) r2 = 1.0;
  else r2 = (-0.0227 * (v) - 1.47);
  x[GO_hf1] = (r1 * (1.0 / (1.0 + exp((v + 72.5) * 0.11))));
  x[GO_hf2] = (r2 * (1.0 / (1.0 + exp((v + 81.9) * 0.16))));
  x[GO_hs1] = ((1.0 - r1) * (1.0 / (1.0 + exp((v + 72.5) * 0.11))));
  x[GO_hs2] = ((1.0 - r2) * (1.0 / (1.0 + exp((v + 81.9) * 0.16))));
  x[GO_o1] = 0.0; x[GO_o2] = 0.0; x[GO_c2] = 0.0; x[GO_c3] = 0.0; x[GO_c4] = 0.0; x[GO_c1] = 1.0;
}

}  // namespace

void initial_state(int type, double jitter, int comp_type, double g_CaH_io, CompInit *out) {
  out->ca2 = 0.0; out->ca_old = 0.0; out->rev = 0.0;
  switch (type) {
    case PKJ:
      out->v = V_INIT_PKJ + 2.0 * jitter;
      out->ca = Ca1_0_PKJ;
      out->rev = V_Ca_PKJ;
      pkj_init(out->v, out->ca, out->x);
      break;
    case IO:
      out->v = V_INIT_IO + 10.0 * jitter;
      io_init(out->v, comp_type, g_CaH_io, &out->ca, out->x);
      break;
    case GR:
      out->v = V_INIT_GR + 2.0 * jitter;
      out->ca = Ca1_0_GR;
      gr_init(out->v, out->ca, out->x);
      break;
    default:
      out->v = V_INIT_GO + 2.0 * jitter;
      out->ca = Ca1_0_GO; out->ca2 = Ca1_0_GO; out->rev = V_Ca_GO; out->ca_old = Ca1_0_GO;
      go_init(out->v, out->ca, out->x);
      break;
  }
}

}  // namespace gbrkc

/*
 * CPU oracle for the RKC hot path -- TEST INFRASTRUCTURE ONLY (see
 * rkc_oracle.h).  Plain FP64, sequential, written to keep the reference's
 * operation order so that the gating kernels agree bit-for-bit with the
 * reference sources compiled for the host.  Compile with -ffp-contract=off.
 *
 * Every function names the reference file:line it restates.
 */
#include "rkc_oracle.h"
#include "canon_math.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* constants (restated from the reference headers)                     */
/* ------------------------------------------------------------------ */
#define H_MAX 0.125                     /* param.h:12, solve_rkc.cuh:23 */
#define UROUND 2.22e-16                 /* solve_rkc.cuh:22 */

/* GR: gr.cuh:15-27 */
#define V_LEAK1_GR (-16.5)
#define V_LEAK2_GR (-65.0)
#define V_LEAK3_GR (-74.5)
#define V_Na_GR 87.39
#define V_K_GR (-84.69)
#define V_Ca_GR 129.33
#define V_INIT_GR (-80.0)
#define Ca1_0_GR 1e-4
/* GO: go.cuh:28-41 */
#define V_INIT_GO (-60.0)
#define V_LEAK_GO (-55.0)
#define V_Na_GO 87.39
#define V_K_GO (-84.69)
#define V_Ca_GO 120.0
#define V_H_GO (-20.0)
#define SHELL1_D_GO 0.2e-4
#define B_Ca1_GO 1.3
#define Ca1_0_GO 5e-5
#define Ca1OUT_GO 2.0
#define F_GO 9.6485e4
#define G_GJ_GO 2.5e-6
/* PKJ: pkj.cuh:20-83 */
#define V_INIT_PKJ (-68.0)
#define V_LEAK_PKJ (-80.0)
#define V_Na_PKJ 45.0
#define V_Ca_PKJ 135.0
#define V_KH_PKJ (-30.0)
#define V_K_PKJ (-85.0)
#define G_GJ_PKJ 2.5e-6
#define PKJ_SPINE_DENS 13.0e4
#define PKJ_SPINE_AREA 1.33e-8
#define PKJ_CM 1.64
#define PKJ_RM_S 10.0
#define PKJ_RM_D 30.0
#define PKJ_RI 0.25
#define B_Ca1_PKJ 10.0
#define PKJ_SHELLD 0.2e-4
#define Ca1OUT_PKJ 2.4
#define Ca1_0_PKJ 4.0e-5
#define F_PKJ 9.6485e4
/* IO: io.cuh:16-51 */
#define V_INIT_IO (-60.0)
#define V_LEAK_IO 10.0
#define V_Na_IO 55.0
#define V_Ca_IO 120.0
#define V_K_IO (-75.0)
#define V_H_IO (-43.0)
#define G_INT_IO 0.13
#define G_P_DS_IO 0.200
#define G_P_SA_IO 0.869
#define G_C_IO 0.04
#define CA_PH_IO 3.0
#define BETA_CA_IO 0.075

/* ion-state / conductance slot orders (gr.cuh:35-41, go.cuh:47-55,
 * pkj.cuh:86-93, io.cuh:56-59) */
enum { GR_n_KV, GR_a_KA, GR_b_KA, GR_c_KCa, GR_s_KM, GR_ir_KIR, GR_ch_Ca, GR_ci_Ca,
       GR_o_Na, GR_c1, GR_c2, GR_c3, GR_c4, GR_c5, GR_i1, GR_i2, GR_i3, GR_i4, GR_i5,
       GR_i6, GR_NION };
enum { GR_g_leak1, GR_g_leak2, GR_g_leak3, GR_g_Na, GR_g_KV, GR_g_KA, GR_g_KCa,
       GR_g_KM, GR_g_KIR, GR_g_Ca, GR_NCOND };
enum { GO_m_NaT, GO_h_NaT, GO_r_NaR, GO_s_NaR, GO_p_NaP, GO_n_KV, GO_a_KA, GO_b_KA,
       GO_c_KC, GO_sl, GO_ch, GO_ci, GO_cl, GO_cm, GO_hf1, GO_hf2, GO_hs1, GO_hs2,
       GO_o1, GO_o2, GO_c1, GO_c2, GO_c3, GO_c4, GO_NION };
enum { GO_g_leak, GO_g_NaT, GO_g_NaR, GO_g_NaP, GO_g_KV, GO_g_KA, GO_g_KC, GO_g_Kslow,
       GO_g_CaHVA, GO_g_CaLVA, GO_g_HCN1, GO_g_HCN2, GO_g_KAHP, GO_NCOND };
enum { PK_m_NaF, PK_h_NaF, PK_m_NaP, PK_m_CaP, PK_h_CaP, PK_m_CaT, PK_h_CaT, PK_m_KA,
       PK_h_KA, PK_m_KC, PK_m_Kh1, PK_m_Kh2, PK_m_Kdr, PK_h_Kdr, PK_m_KM, PK_z_KC,
       PK_m_K2, PK_z_K2, PK_NION };
enum { PK_g_leak, PK_g_NaF, PK_g_NaP, PK_g_CaP, PK_g_CaT, PK_g_Kh, PK_g_Kdr, PK_g_KM,
       PK_g_KA, PK_g_KC, PK_g_K2, PK_NCOND };
enum { IO_k, IO_l, IO_m, IO_h, IO_n, IO_p, IO_x, IO_r, IO_s, IO_q, IO_NION };
enum { IO_g_leak, IO_g_CaL, IO_g_Na, IO_g_Kdr, IO_g_K, IO_g_CaH, IO_g_KCa, IO_g_H, IO_NCOND };

/* logical RKC vectors (param.h:21) mapped onto physical buffers */
enum { LY, LYN, LFN, LV1, LV2, NLOG };

struct orc_sys {
  int type, nx, ny, n, ncomp, nc;
  /* elem (param.h:20) */
  double *v, *ca, *cm, *area, *compart, *iext;
  double *cond[16];
  double *ion[24];
  int ncond, nion;
  double *ca2, *rev_ca2, *ca_old, *shell;
  int *rev_fixed; /* PKJ Nernst quirk: global id % 1599 == 0 (pkj_ion.cu:329) */
  /* CSR (RKC sign convention: off-diagonals +g, diagonal kept) */
  int nnz;
  double *val;
  int *col, *row;
  double *b;
  /* RKC vectors */
  double *phys[NLOG];
  int map[NLOG];
  double *ede, *vnew, *dammy;
  /* controller (param.h:22, h_work/h_others/h_bool of solve_rkc.cu) */
  double mmax, absh, sprad, naccpt, atol, rtol, idid, gt, gt_old, lt, tend, errold,
      hold, nstsig;
  double cbrt_errold; /* canonical mode: errold^(1/3) kept from the last accepted step */
  double hw[8];
  int last, newspc, jacatt;
  double sum_dt, integ;
  double hmin;
  /* stimulus */
  int *stim_comp;
  double *stim_amp, *stim_t0, *stim_t1;
  /* IO gap: 4 directed edges per cell (gap.cu:4-120) */
  int ngap;
  int *gap_pre, *gap_post;
  double *gap_cur, *gap_g;
  int canon;
  double *invcm, *scratch;
  /* counters */
  long long n_steps, n_rej, n_stage, n_rho, n_ion, n_rho_iter;
  /* chemical synapses onto this system (network mode, set by orc_net_build):
   * 1 = g (V_y - E) per synapse at each ion update (granule), 2 = the sum taken
   * at interval start added at each ion update (Golgi), 3 = as 2 scaled by
   * exp(-sum_dt / 0.6) (Purkinje) -- solve_rkc.cu:198-360, 1100-1120, 1180-1270 */
  int syn_mode;
  int *syn_row, *syn_idx;   /* CSR over compartments: synapse ids in (kind, id) order */
  const double *syn_val, *syn_e;
  double *syn_buf;
};

#define VEC(s, L) ((s)->phys[(s)->map[L]])

/* Canonical mode (see canon_math.h): the platform exp/log/pow are replaced by
 * the agreed implementations, the vector updates use the GPU path's explicit
 * fused multiply-adds, 1/Cm is a multiply, and every sum is the pairwise
 * tree below.  Reference mode keeps the reference's literal expressions. */
static int g_canon = 0;
#define EXP(x) (g_canon ? cm_exp(x) : exp(x))
#define LOG(x) (g_canon ? cm_log(x) : log(x))
#define POW(x, y) (g_canon ? cm_pow((x), (y)) : pow((x), (y)))

/* pairwise tree over indices 0..n-1 (stride doubling, in place) */
static double tree_sum(double *a, int n) {
  if (n <= 0) return 0.0;
  for (int stride = 1; stride < n; stride *= 2)
    for (int i = 0; i + stride < n; i += 2 * stride) a[i] = a[i] + a[i + stride];
  return a[0];
}

static double *zalloc(size_t n) { return (double *)calloc(n ? n : 1, sizeof(double)); }
static int *ialloc(size_t n) { return (int *)calloc(n ? n : 1, sizeof(int)); }

int orc_row_fields(int type) {
  switch (type) {
    case ORC_GR: return 17;
    case ORC_GO: return 20;
    case ORC_PKJ: return 7;
    case ORC_IO: return 6;
  }
  return 0;
}

/* ------------------------------------------------------------------ */
/* PKJ rate functions (pkj_ion.cu:4-91)                                 */
/* ------------------------------------------------------------------ */
static double pk_l(double v, double A, double B, double C, double D) {
  return A / (B + EXP((v + C) / D));
}
static double pk_am_NaF(double v) { return pk_l(v, 35.0, 0.0, 5.0, -10.0); }
static double pk_ah_NaF(double v) { return pk_l(v, 0.225, 1.0, 80.0, 10.0); }
static double pk_am_NaP(double v) { return pk_l(v, 200.0, 1.0, -18.0, -16.0); }
static double pk_am_CaP(double v) { return pk_l(v, 8.5, 1.0, -8.0, -12.5); }
static double pk_ah_CaP(double v) { return pk_l(v, 0.0015, 1.0, 29.0, 8.0); }
static double pk_am_CaT(double v) { return pk_l(v, 2.60, 1.0, 21.0, -8.0); }
static double pk_ah_CaT(double v) { return pk_l(v, 0.0025, 1.0, 40.0, 8.0); }
static double pk_am_KA(double v) { return pk_l(v, 1.40, 1.0, 27.0, -12.0); }
static double pk_ah_KA(double v) { return pk_l(v, 0.0175, 1.0, 50.0, 8.0); }
static double pk_bm_NaF(double v) { return pk_l(v, 7.0, 0.0, 65.0, 20.0); }
static double pk_bh_NaF(double v) { return pk_l(v, 7.5, 0.0, -3.0, -18.0); }
static double pk_bm_NaP(double v) { return pk_l(v, 25.0, 1.0, 58.0, 8.0); }
static double pk_bm_CaP(double v) { return pk_l(v, 35.0, 1.0, 74.0, 14.5); }
static double pk_bh_CaP(double v) { return pk_l(v, 0.0055, 1.0, 23.0, -8.0); }
static double pk_bm_CaT(double v) { return pk_l(v, 0.180, 1.0, 40.0, 4.0); }
static double pk_bh_CaT(double v) { return pk_l(v, 0.190, 1.0, 50.0, -10.0); }
static double pk_bm_KA(double v) { return pk_l(v, 0.490, 1.0, 30.0, 4.0); }
static double pk_bh_KA(double v) { return pk_l(v, 1.30, 1.0, 13.0, -10.0); }
static double pk_bm_KC(double v) { return pk_l(v, 0.110, 0.0, -35.0, 14.9); }
static double pk_bm_K2(double v) { return pk_l(v, 0.075, 0.0, 25.0, 6.0); }

/* a generic alpha/beta gate: inf = a/(a+b), tau = 1/(a+b) */
#define AB_GATE(name, afn, bfn)                                                      \
  static double name##_inf(double v) { return afn(v) / (afn(v) + bfn(v)); }          \
  static double name##_tau(double v) { return 1.0 / (afn(v) + bfn(v)); }

AB_GATE(pk_m_NaF, pk_am_NaF, pk_bm_NaF)
AB_GATE(pk_h_NaF, pk_ah_NaF, pk_bh_NaF)
AB_GATE(pk_m_NaP, pk_am_NaP, pk_bm_NaP)
AB_GATE(pk_m_CaP, pk_am_CaP, pk_bm_CaP)
AB_GATE(pk_h_CaP, pk_ah_CaP, pk_bh_CaP)
AB_GATE(pk_m_CaT, pk_am_CaT, pk_bm_CaT)
AB_GATE(pk_h_CaT, pk_ah_CaT, pk_bh_CaT)
AB_GATE(pk_m_KA, pk_am_KA, pk_bm_KA)
AB_GATE(pk_h_KA, pk_ah_KA, pk_bh_KA)

static double pk_m_KC_inf(double v) { return 7.5 / (7.5 + pk_bm_KC(v)); }
static double pk_m_KC_tau(double v) { return 1.0 / (7.5 + pk_bm_KC(v)); }
static double pk_m_K2_inf(double v) { return 25.0 / (25.0 + pk_bm_K2(v)); }
static double pk_m_K2_tau(double v) { return 1.0 / (25.0 + pk_bm_K2(v)); }
static double pk_m_Kh1_inf(double v) { return 0.8 / (1.0 + EXP((v + 82.0) / 7.0)); }
static double pk_m_Kh2_inf(double v) { return 0.2 / (1.0 + EXP((v + 82.0) / 7.0)); }
static double pk_m_Kdr_tau(double v) {
  double a;
  if (fabs(v + 12.0) > 1e-6) a = -0.0235 * (v + 12.0) / (EXP(-(v + 12.0) / 12.0) - 1.0);
  else a = 0.0235 * 12.0;
  double b = 5.0 * EXP(-(v + 147.0) / 30.0);
  return 1.0 / (a + b);
}
static double pk_m_Kdr_inf(double v) {
  double a;
  if (fabs(v - 8.0) > 1e-6) a = -0.0235 * (v - 8.0) / (EXP(-(v - 8.0) / 12.0) - 1.0);
  else a = 0.0235 * 12.0;
  double b = 5.0 * EXP(-(v + 127.0) / 30.0);
  return a / (a + b);
}
static double pk_h_Kdr_tau(double v) { return (v < -25.0) ? 1200.0 : 10.0; }
static double pk_h_Kdr_inf(double v) { return 1.0 / (1.0 + EXP((v + 25.0) / 4.0)); }
static double pk_m_KM_tau(double v) {
  return 200.0 / (3.3 * (EXP((v + 35.0) / 20.0)) + EXP(-(v + 35.0) / 20.0));
}
static double pk_m_KM_inf(double v) { return 1.0 / (1.0 + EXP(-(v + 35.0) / 10.0)); }
static double pk_z_KC_inf(double ca) { return 1.0 / (1.0 + 4.00 / ca); }
static double pk_z_K2_inf(double ca) { return 1.0 / (1.0 + 0.20 / ca); }

/* trapezoid gate step used by every *_update_ion_RKC kernel */
static double trap(double dt, double inf, double tau, double x) {
  return (2.0 * dt * inf + (2.0 * tau - dt) * x) / (2.0 * tau + dt);
}

/* ------------------------------------------------------------------ */
/* IO rate functions (io_ion.cu:5-51)                                  */
/* ------------------------------------------------------------------ */
static double io_ar(double v) { return (1.7) / (1.0 + EXP((-(v - 5.0)) / 13.9)); }
static double io_as(double x) { return fmin(0.00002 * x, 0.01); }
static double io_ax(double v) { return (0.13 * (v + 25.0)) / (1.0 - EXP(-(v + 25.0) / 10.0)); }
static double io_br(double v) { return (0.02 * (v + 8.5)) / (EXP((v + 8.5) / 5.0) - 1.0); }
static double io_bx(double v) { return 1.69 * EXP(-0.0125 * (v + 35.0)); }
static double io_h_inf(double v, int e) {
  double h = 1.0;
  if (e == 1) h = 1.0 / (1.0 + EXP((-v - 70.0) / (-5.8)));
  if (e == 2) h = 1.0 / (1.0 + EXP((-v - 60.0) / (-5.8)));
  return h;
}
static double io_k_inf(double v) { return 1.0 / (1.0 + EXP((-v - 61.0) / 4.2)); }
static double io_l_inf(double v) { return 1.0 / (1.0 + EXP((v + 85.5) / (8.5))); }
static double io_m_inf(double v) { return 1.0 / (1.0 + EXP((-v - 30.0) / (5.5))); }
static double io_n_inf(double v) { return 1.0 / (1.0 + EXP((-v - 3.0) / (10.0))); }
static double io_p_inf(double v) { return 1.0 / (1.0 + EXP((-v - 51.0) / (-12.0))); }
static double io_q_inf(double v) { return 1.0 / (1.0 + EXP((v + 80.0) / 4.0)); }
static double io_r_inf(double v) { return io_ar(v) / (io_ar(v) + io_br(v)); }
static double io_s_inf(double x) { return io_as(x) / (io_as(x) + 0.015); }
static double io_x_inf(double v) { return io_ax(v) / (io_ax(v) + io_bx(v)); }
static double io_h_tau(double v, int e) {
  double h = 1.0;
  if (e == 1) h = 3.0 * EXP((-v - 40.0) / 33.0);
  if (e == 2) h = 1.5 * EXP((-v - 40.0) / 33.0);
  return h;
}
static double io_l_tau(double v) {
  return ((20.0 * EXP((v + 160.0) / 30.0)) / (1.0 + EXP((v + 84.0) / 7.3))) + 35.0;
}
static double io_n_tau(double v) { return 47.0 * EXP((-(-v - 50.0)) / 900.0) + 5.0; }
static double io_q_tau(double v) { return 1.0 / (EXP(-0.086 * v - 14.6) + EXP(0.07 * v - 1.87)); }
static double io_r_tau(double v) { return 5.0 / (io_ar(v) + io_br(v)); }
static double io_s_tau(double x) { return 1.0 / (io_as(x) + 0.015); }
static double io_x_tau(double v) { return 1.0 / (io_ax(v) + io_bx(v)); }

/* ------------------------------------------------------------------ */
/* GR rate functions (gr_ion.cu:3-43)                                  */
/* ------------------------------------------------------------------ */
static double gr_a_nKV(double v) {
  return (fabs(v + 25.0) > 1.0e-6) ? -0.017 * ((v + 25.0) / (EXP(-(v + 25.0) / 10.0) - 1.0))
                                   : -0.17 * (1.0 + (v + 25.0) / 20.0);
}
static double gr_b_nKV(double v) { return 0.2223 * EXP(-(v + 35.0) / 80.0); }
AB_GATE(gr_nKV, gr_a_nKV, gr_b_nKV)
static double gr_a_aKA(double v) { return 0.771 / (1.0 + EXP(-(v + 9.17203) / 23.32708)); }
static double gr_b_aKA(double v) { return 0.1567 / EXP((v + 18.27914) / 19.47175); }
static double gr_aKA_inf(double v) { return 1.0 / (1.0 + EXP(-(v + 38.0) / 17.0)); }
static double gr_aKA_tau(double v) { return (1.0 / (gr_a_aKA(v) + gr_b_aKA(v))); }
static double gr_a_bKA(double v) { return 0.0348 / (1.0 + EXP((v + 111.33208) / 12.8433)); }
static double gr_b_bKA(double v) { return 0.0327 / (1.0 + EXP(-(v + 49.9537) / 8.90123)); }
static double gr_bKA_inf(double v) { return 1.0 / (1.0 + EXP((v + 78.8) / 8.4)); }
static double gr_bKA_tau(double v) { return (1.0 / (gr_a_bKA(v) + gr_b_bKA(v))); }
static double gr_a_ir(double v) { return 0.2302 * EXP(-(v + 83.94) / 24.3902); }
static double gr_b_ir(double v) { return 0.2943 * EXP((v + 83.94) / 35.714); }
AB_GATE(gr_ir, gr_a_ir, gr_b_ir)
static double gr_a_sKM(double v) { return 0.0046 * EXP((v + 30.0) / 40.0); }
static double gr_b_sKM(double v) { return 0.0046 * EXP(-(v + 30.0) / 20.0); }
static double gr_sKM_inf(double v) { return 1.0 / (1.0 + EXP(-(v + 35.0) / 6.0)); }
static double gr_sKM_tau(double v) { return (1.0 / (gr_a_sKM(v) + gr_b_sKM(v))); }
static double gr_a_cKCa(double v, double ca) { return 1.4433 / (1.0 + (1.5e-3 * EXP(-v / 11.765)) / ca); }
static double gr_b_cKCa(double v, double ca) { return 0.8660 / (1.0 + ca / (1.5e-4 * EXP(-v / 11.765))); }
static double gr_cKCa_inf(double v, double ca) {
  return gr_a_cKCa(v, ca) / (gr_a_cKCa(v, ca) + gr_b_cKCa(v, ca));
}
static double gr_cKCa_tau(double v, double ca) { return (1.0 / (gr_a_cKCa(v, ca) + gr_b_cKCa(v, ca))); }
static double gr_a_ch(double v) { return 0.0856 * EXP((v + 29.6) / 15.873); }
static double gr_b_ch(double v) { return 0.1437 * EXP(-(v + 18.66) / 25.641); }
static double gr_a_ci(double v) { return 0.0023 * EXP(-(v + 48.0) / 18.183); }
static double gr_b_ci(double v) { return 0.0025 * EXP((v + 48.0) / 83.33); }
static double gr_ch_inf(double v) { return (gr_a_ch(v) / (gr_a_ch(v) + gr_b_ch(v))); }
static double gr_ci_inf(double v) { return (gr_a_ci(v) / (gr_a_ci(v) + gr_b_ci(v))); }

/* ------------------------------------------------------------------ */
/* GO rate functions (go_ion.cu:3-86)                                  */
/* ------------------------------------------------------------------ */
static double go_am_NaT(double v) { return 0.417 * (v + 25.0) / (1 - EXP(-(v + 25.0) / 10.0)); }
static double go_bm_NaT(double v) { return 16.68 * EXP(-0.055 * (v + 50.0)); }
AB_GATE(go_m_NaT, go_am_NaT, go_bm_NaT)
static double go_ah_NaT(double v) { return 0.292 * EXP(-0.3 * (v + 50.0)); }
static double go_bh_NaT(double v) { return 4.17 / (1 + EXP(-(v + 17.0) / 5.0)); }
AB_GATE(go_h_NaT, go_ah_NaT, go_bh_NaT)
static double go_ar_NaR(double v) {
  return ((1.11 - 68.5 * (v - 4.48) / (EXP(-(v - 4.48) / 6.8) - 1.0)) * 1.0e-4);
}
static double go_br_NaR(double v) {
  double x = (v + 44.0) / 0.11;
  if (x > 200.0) x = 200.0;
  return ((66.0 + 21.7 * (v + 44) / (EXP(x) - 1.0)) * 1.0e-3);
}
AB_GATE(go_r_NaR, go_ar_NaR, go_br_NaR)
static double go_as_NaR(double v) { return (0.443 * EXP(-(v + 80.0) / 62.5)); }
static double go_bs_NaR(double v) { return (0.014 * EXP((v + 83.3) / 16.1)); }
AB_GATE(go_s_NaR, go_as_NaR, go_bs_NaR)
static double go_ap_NaP(double v) { return (0.421 * (v + 40.0) / (1.0 - EXP(-(v + 40.0) / 5.0))); }
static double go_bp_NaP(double v) { return (-0.287 * (v + 40.0) / (1.0 - EXP((v + 40.0) / 5.0))); }
static double go_p_NaP_inf(double v) { return (1 / (1.0 + EXP(-(v + 43.0) / 5.0))); }
static double go_p_NaP_tau(double v) { return (5.0 / (go_ap_NaP(v) + go_bp_NaP(v))); }
static double go_ach(double v) { return (0.0687 * EXP(0.063 * (v + 29.0))); }
static double go_bch(double v) { return (0.115 * EXP(-0.039 * (v + 18.66))); }
AB_GATE(go_ch, go_ach, go_bch)
static double go_aci(double v) { return (1.8e-3 * EXP(-(v + 48.0) / 18.0)); }
static double go_bci(double v) { return (1.8e-3 * EXP((v + 48.0) / 83.0)); }
AB_GATE(go_ci, go_aci, go_bci)
static double go_cl_inf(double v) { return (1.0 / (1.0 + EXP(-(v + 52.0) / 7.4))); }
static double go_cl_tau(double v) {
  return ((3.0 + 1.0 / (EXP((v + 27.0) / 10.0) + EXP(-(v + 102.0) / 15.0))) / 0.85);
}
static double go_cm_inf(double v) { return (1.0 / (1.0 + EXP((v + 80.0) / 5.0))); }
static double go_cm_tau(double v) {
  return ((85.0 + 1.0 / (EXP((v + 48.0) / 4.0) + EXP(-(v + 407.0) / 50.0))) / 0.9);
}
static double go_an_KV(double v) { return 0.062 * (v + 26.0) / (1.0 - EXP(-(v + 26.0) / 10.0)); }
static double go_bn_KV(double v) { return 0.78 * EXP(-(v + 36.0) / 80.0); }
AB_GATE(go_n_KV, go_an_KV, go_bn_KV)
static double go_aa_KA(double v) { return (0.62 / (1.0 + EXP(-(v + 9.17) / 23.32))); }
static double go_ba_KA(double v) { return (0.126 / (EXP((v + 18.28) / 19.47))); }
static double go_a_KA_inf(double v) { return (1.0 / (1.0 + EXP(-(v + 38.0) / 17.0))); }
static double go_a_KA_tau(double v) { return (1.0 / (go_aa_KA(v) + go_ba_KA(v))); }
static double go_ab_KA(double v) { return (0.028 / (1.0 + EXP((v + 111.0) / 12.84))); }
static double go_bb_KA(double v) { return (0.026 / (1.0 + EXP(-(v + 49.95) / 8.9))); }
static double go_b_KA_inf(double v) { return (1.0 / (1.0 + EXP((v + 78.8) / 8.4))); }
static double go_b_KA_tau(double v) { return (1.0 / (go_ab_KA(v) + go_bb_KA(v))); }
static double go_ac_KC(double v, double ca) { return (3.2 / (1.0 + 0.0015 * EXP(-(v) / 11.7) / ca)); }
static double go_bc_KC(double v, double ca) { return (0.46 / (1.0 + ca / (1.5e-4 * EXP(-(v) / 11.7)))); }
static double go_c_KC_inf(double v, double ca) {
  return (go_ac_KC(v, ca) / (go_ac_KC(v, ca) + go_bc_KC(v, ca)));
}
static double go_c_KC_tau(double v, double ca) { return (1.0 / (go_ac_KC(v, ca) + go_bc_KC(v, ca))); }
static double go_asl(double v) { return (0.0037 * EXP((v + 30.0) / 40.0)); }
static double go_bsl(double v) { return (0.0037 * EXP(-(v + 30.0) / 20.0)); }
static double go_sl_inf(double v) { return (1.0 / (1.0 + EXP(-(v + 35.0) / 6.0))); }
static double go_sl_tau(double v) { return (1.0 / (go_asl(v) + go_bsl(v))); }
static double go_r1(double v) { return (0.0021 * (v) + 0.97); }
static double go_hf1_inf(double v) { return (go_r1(v) * (1.0 / (1.0 + EXP((v + 72.5) * 0.11)))); }
static double go_hs1_inf(double v) { return ((1.0 - go_r1(v)) * (1.0 / (1.0 + EXP((v + 72.5) * 0.11)))); }
static double go_hf1_tau(double v) { return (EXP((0.0137 * v + 3.37) * 2.3)); }
static double go_hs1_tau(double v) { return (EXP((0.0145 * v + 4.06) * 2.3)); }
static double go_r2(double v) {
  if (v >= -64.70) return 0.0;
  else if (v <= -108.70) return 1.0;
  else return (-0.0227 * (v) - 1.47);
}
static double go_hf2_inf(double v) { return (go_r2(v) * (1.0 / (1.0 + EXP((v + 81.9) * 0.16)))); }
static double go_hs2_inf(double v) { return ((1.0 - go_r2(v)) * (1.0 / (1.0 + EXP((v + 81.9) * 0.16)))); }
static double go_hf2_tau(double v) { return (EXP((0.027 * v + 5.6) * 2.3)); }
static double go_hs2_tau(double v) { return (EXP((0.015 * v + 5.3) * 2.3)); }

/* ------------------------------------------------------------------ */
/* small dense solver: partial pivoting Gaussian elimination as in      */
/* gr_ion.cu:141-190 and go_ion.cu:152-200.  Returns 0 on a "pivot     */
/* error" (the reference returns early and leaves the state).          */
/* ------------------------------------------------------------------ */
/* Row swaps taken over the process's lifetime: the kinetic matrices are
 * strictly column diagonally dominant, so this stays zero (the CUDA path
 * relies on it and the tests check it). */
static long long g_pivot_swaps = 0;
long long orc_pivot_swaps(void) { return g_pivot_swaps; }

/* the canonical exp / log / pow, exported for tests/test_canon_math.py */
double orc_cm_exp(double x) { return cm_exp(x); }
double orc_cm_log(double x) { return cm_log(x); }
double orc_cm_pow(double x, double y) { return cm_pow(x, y); }
double orc_cm_cbrt(double x) { return cm_cbrt(x); }

static int pivot_solve(int n, double *A /* n*n row-major */, double *bvec) {
  for (int i = 0; i < n - 1; i++) {
    int piv = i;
    double pmax = fabs(A[i * n + i]);
    for (int j = i + 1; j < n; j++)
      if (fabs(A[j * n + i]) > pmax) { piv = j; pmax = fabs(A[j * n + i]); }
    if (fabs(pmax) < 1.0e-12) return 0;
    if (piv != i) {
      g_pivot_swaps++;
      for (int j = i; j < n; j++) {
        double t = A[i * n + j]; A[i * n + j] = A[piv * n + j]; A[piv * n + j] = t;
      }
      double t = bvec[i]; bvec[i] = bvec[piv]; bvec[piv] = t;
    }
    for (int j = i + 1; j < n; j++) {
      double w = A[j * n + i] / A[i * n + i];
      A[j * n + i] = 0.0;
      for (int k = i + 1; k < n; k++) A[j * n + k] = A[j * n + k] - A[i * n + k] * w;
      bvec[j] = bvec[j] - bvec[i] * w;
    }
  }
  for (int i = n - 1; i >= 0; i--) {
    for (int j = i + 1; j < n; j++) {
      bvec[i] = bvec[i] - A[i * n + j] * bvec[j];
      A[i * n + j] = 0.0;
    }
    bvec[i] = bvec[i] / A[i * n + i];
    A[i * n + i] = 1.0;
  }
  return 1;
}

/* GR 12-state Na channel, Crank-Nicolson step (gr_ion.cu:45-207).
 * Per-compartment-type parameters for types 5..8 (hillock, AIS, axon, pf). */
static const double GRNA_n1[9] = {1, 1, 1, 1, 1, 5.422, 5.422, 5.422, 5.422};
static const double GRNA_n2[9] = {1, 1, 1, 1, 1, 3.279, 3.279, 3.279, 3.279};
static const double GRNA_n3[9] = {1, 1, 1, 1, 1, 1.83, 1.83, 1.83, 1.83};
static const double GRNA_n4[9] = {1, 1, 1, 1, 1, 0.738, 0.738, 0.738, 0.738};
static const double GRNA_Aa[9] = {1, 1, 1, 1, 1, 8.85, 8.85, 8.85, 8.85};
static const double GRNA_Ab[9] = {1, 1, 1, 1, 1, 0.0318, 0.0318, 0.0318, 0.0318};
static const double GRNA_Vs[9] = {1, 1, 1, 1, 1, -22.0, -22.0, -25.0, -25.0};
static const double GRNA_Con[9] = {1, 1, 1, 1, 1, 0.003464, 0.003464, 0.09353, 0.09353};
static const double GRNA_Coff[9] = {1, 1, 1, 1, 1, 0.4157, 0.4157, 0.04676, 0.04676};
static const double GRNA_Oon[9] = {1, 1, 1, 1, 1, 1.8186, 1.8186, 2.5981, 2.5981};
static const double GRNA_Ooff[9] = {1, 1, 1, 1, 1, 0.006928, 0.006928, 0.000173, 0.000173};

/* Fill the 12x12 Na kinetic matrix; sgn = -1 for the explicit half
 * (diagonal "- 2/DT"), +1 for the implicit half ("+ 2/DT"). */
static void grna_matrix(double M[144], int t, double alpha, double beta, double DT, double sgn) {
  const double n1 = GRNA_n1[t], n2 = GRNA_n2[t], n3 = GRNA_n3[t], n4 = GRNA_n4[t];
  const double Con = GRNA_Con[t], Coff = GRNA_Coff[t], Oon = GRNA_Oon[t], Ooff = GRNA_Ooff[t];
  const double a = pow((GRNA_Oon[t] / GRNA_Con[t]), 0.25);
  const double b = pow((GRNA_Ooff[t] / GRNA_Coff[t]), 0.25);
  const double tdt = 2.0 / DT;
  for (int i = 0; i < 144; i++) M[i] = 0.0;
#define S(r, c, x) M[(r)*12 + (c)] = (x)
  /* the diagonal terms are -(rates + sgn*2/DT) */
  if (sgn < 0) {
    S(0, 0, -(n1 * alpha + Con - tdt));
    S(1, 1, -(n4 * beta + n2 * alpha + Con * a - tdt));
    S(2, 2, -(n3 * beta + n3 * alpha + Con * a * a - tdt));
    S(3, 3, -(n2 * beta + n4 * alpha + Con * a * a * a - tdt));
    S(4, 4, -(n1 * beta + 259.8 + Con * pow(a, 4.0) - tdt));
    S(5, 5, -(Coff + n1 * alpha * a - tdt));
    S(6, 6, -(Coff * b + n4 * beta * b + n2 * alpha * a - tdt));
    S(7, 7, -(Coff * b * b + n3 * beta * b + n3 * alpha * a - tdt));
    S(8, 8, -(Coff * b * b * b + n2 * beta * b + n4 * alpha * a - tdt));
    S(9, 9, -(Coff * pow(b, 4.0) + n1 * beta * b + 259.8 - tdt));
    S(10, 10, -(Ooff + 69.3 - tdt));
    S(11, 11, -(69.3 + Oon - tdt));
  } else {
    S(0, 0, -(n1 * alpha + Con + tdt));
    S(1, 1, -(n4 * beta + n2 * alpha + Con * a + tdt));
    S(2, 2, -(n3 * beta + n3 * alpha + Con * a * a + tdt));
    S(3, 3, -(n2 * beta + n4 * alpha + Con * a * a * a + tdt));
    S(4, 4, -(n1 * beta + 259.8 + Con * pow(a, 4.0) + tdt));
    S(5, 5, -(Coff + n1 * alpha * a + tdt));
    S(6, 6, -(Coff * b + n4 * beta * b + n2 * alpha * a + tdt));
    S(7, 7, -(Coff * b * b + n3 * beta * b + n3 * alpha * a + tdt));
    S(8, 8, -(Coff * b * b * b + n2 * beta * b + n4 * alpha * a + tdt));
    S(9, 9, -(Coff * pow(b, 4.0) + n1 * beta * b + 259.8 + tdt));
    S(10, 10, -(Ooff + 69.3 + tdt));
    S(11, 11, -(69.3 + Oon + tdt));
  }
  S(0, 1, n4 * beta); S(0, 5, Coff);
  S(1, 0, n1 * alpha); S(1, 2, n3 * beta); S(1, 6, Coff * b);
  S(2, 1, n2 * alpha); S(2, 3, n2 * beta); S(2, 7, Coff * b * b);
  S(3, 2, n3 * alpha); S(3, 4, n1 * beta); S(3, 8, Coff * b * b * b);
  S(4, 3, n4 * alpha); S(4, 9, Coff * pow(b, 4.0)); S(4, 11, 69.3);
  S(5, 0, Con); S(5, 6, n4 * beta * b);
  S(6, 1, Con * a); S(6, 5, n1 * alpha * a); S(6, 7, n3 * beta * b);
  S(7, 2, Con * a * a); S(7, 6, n2 * alpha * a); S(7, 8, n2 * beta * b);
  S(8, 3, Con * a * a * a); S(8, 7, n3 * alpha * a); S(8, 9, n1 * beta * b);
  S(9, 4, Con * pow(a, 4.0)); S(9, 8, n4 * alpha * a); S(9, 10, 69.3);
  S(10, 9, 259.8); S(10, 11, Oon);
  S(11, 4, 259.8); S(11, 10, Ooff);
#undef S
}

static void gr_na_update(orc_sys *s, int id, double v_new, double v_old, double DT) {
  int t = (int)s->compart[id];
  if (t < 5) return; /* GR_hill = 5 */
  const double vs = GRNA_Vs[t];
  double M[144], vc[12], vcb[12];
  double alpha = GRNA_Aa[t] * EXP((v_old - vs) / 10.0);
  double beta = GRNA_Ab[t] * EXP(-(v_old - vs) / 10.0);
  grna_matrix(M, t, alpha, beta, DT, -1.0);
  static const int slot[12] = {GR_c1, GR_c2, GR_c3, GR_c4, GR_c5, GR_i1,
                               GR_i2, GR_i3, GR_i4, GR_i5, GR_i6, GR_o_Na};
  for (int k = 0; k < 12; k++) vc[k] = s->ion[slot[k]][id];
  for (int i = 0; i < 12; i++) {
    vcb[i] = 0.0;
    for (int j = 0; j < 12; j++) vcb[i] -= vc[j] * M[i * 12 + j];
  }
  alpha = GRNA_Aa[t] * EXP((v_new - vs) / 10.0);
  beta = GRNA_Ab[t] * EXP(-(v_new - vs) / 10.0);
  grna_matrix(M, t, alpha, beta, DT, +1.0);
  if (!pivot_solve(12, M, vcb)) return;
  for (int k = 0; k < 12; k++) s->ion[slot[k]][id] = vcb[k];
}

/* GO 6-state KAHP, Crank-Nicolson step (go_ion.cu:88-213) */
static void go_kahp_update(orc_sys *s, int id, double DT) {
  const double i1 = 80e-3, i2 = 80e-3, i3 = 200e-3, a1 = 1.0, a2 = 100e-3, b1 = 160e-3, b2 = 1.2;
  double l_ca = s->ca_old[id];
  s->ca_old[id] = s->ca[id];
  double l_dt = 2.0 / DT;
  double d1 = 200 * l_ca / 3.0, d2 = 160 * l_ca / 3.0, d3 = 80 * l_ca / 3.0;
  double M[36], vc[6], vcb[6];
  double E[36] = {-d1 + l_dt, i1, 0.0, 0.0, 0.0, 0.0,
                  d1, -d2 - i1 + l_dt, i2, 0.0, 0.0, 0.0,
                  0.0, d2, -(d3 + i2 + b1) + l_dt, i3, a1, 0.0,
                  0.0, 0.0, d3, -(i3 + b2) + l_dt, 0.0, a2,
                  0.0, 0.0, b1, 0.0, -a1 + l_dt, 0.0,
                  0.0, 0.0, 0.0, b2, 0.0, -a2 + l_dt};
  static const int slot[6] = {GO_c1, GO_c2, GO_c3, GO_c4, GO_o1, GO_o2};
  for (int k = 0; k < 6; k++) vc[k] = s->ion[slot[k]][id];
  for (int i = 0; i < 6; i++) {
    vcb[i] = 0.0;
    for (int j = 0; j < 6; j++) vcb[i] -= vc[j] * E[i * 6 + j];
  }
  l_ca = s->ca[id];
  d1 = 200 * l_ca / 3.0; d2 = 160 * l_ca / 3.0; d3 = 80 * l_ca / 3.0;
  double I[36] = {-d1 - l_dt, i1, 0.0, 0.0, 0.0, 0.0,
                  d1, -d2 - i1 - l_dt, i2, 0.0, 0.0, 0.0,
                  0.0, d2, -(d3 + i2 + b1) - l_dt, i3, a1, 0.0,
                  0.0, 0.0, d3, -(i3 + b2) - l_dt, 0.0, a2,
                  0.0, 0.0, b1, 0.0, -a1 - l_dt, 0.0,
                  0.0, 0.0, 0.0, b2, 0.0, -a2 - l_dt};
  memcpy(M, I, sizeof M);
  if (!pivot_solve(6, M, vcb)) return;
  for (int k = 0; k < 6; k++) s->ion[slot[k]][id] = vcb[k];
}

/* ------------------------------------------------------------------ */
/* RKC ion updates per type                                            */
/* ------------------------------------------------------------------ */
/* pkj_update_ion_RKC (pkj_ion.cu:304-358) */
static void pkj_ion_one(orc_sys *s, int id, double vnew, double DT) {
  double **x = s->ion;
  double v_old = s->v[id];
  double v_val = 0.5 * (vnew + v_old);
  double Ca_val = s->ca[id];
  double I = 1e-3 * (v_old - s->rev_ca2[id]) *
             (s->cond[PK_g_CaP][id] * x[PK_m_CaP][id] * x[PK_h_CaP][id] +
              s->cond[PK_g_CaT][id] * x[PK_m_CaT][id] * x[PK_h_CaT][id]);
  if (I > 0.0) I = 0.0;
  else I = -I / (2.0 * F_PKJ * s->shell[id]);
  double k1 = DT * (I - B_Ca1_PKJ * (Ca_val - Ca1_0_PKJ));
  double k2 = DT * (I - B_Ca1_PKJ * (Ca_val + k1 / 2.0 - Ca1_0_PKJ));
  double k3 = DT * (I - B_Ca1_PKJ * (Ca_val + k2 / 2.0 - Ca1_0_PKJ));
  double k4 = DT * (I - B_Ca1_PKJ * (Ca_val + k3 - Ca1_0_PKJ));
  k1 = Ca_val + (k1 + k2 * 2.0 + k3 * 2.0 + k4) / 6.0;
  s->ca[id] = k1;
  Ca_val = 0.5 * (Ca_val + k1);
  if (s->rev_fixed[id]) s->rev_ca2[id] = 12.5 * LOG(Ca1OUT_PKJ / Ca1_0_PKJ);
  else s->rev_ca2[id] = 13.361624877 * LOG(Ca1OUT_PKJ / Ca_val);
  Ca_val = floor((Ca_val * 1000 - 0.04) / 0.099986667) * 0.099986667 + 0.04;
#define G(k, name) x[k][id] = trap(DT, name##_inf(v_val), name##_tau(v_val), x[k][id])
  G(PK_m_NaF, pk_m_NaF); G(PK_h_NaF, pk_h_NaF); G(PK_m_NaP, pk_m_NaP);
  G(PK_m_CaP, pk_m_CaP); G(PK_h_CaP, pk_h_CaP); G(PK_m_CaT, pk_m_CaT);
  G(PK_h_CaT, pk_h_CaT);
  x[PK_m_Kh1][id] = trap(DT, pk_m_Kh1_inf(v_val), 7.6, x[PK_m_Kh1][id]);
  x[PK_m_Kh2][id] = trap(DT, pk_m_Kh2_inf(v_val), 36.8, x[PK_m_Kh2][id]);
  G(PK_m_Kdr, pk_m_Kdr); G(PK_h_Kdr, pk_h_Kdr); G(PK_m_KM, pk_m_KM);
  G(PK_m_KA, pk_m_KA); G(PK_h_KA, pk_h_KA); G(PK_m_KC, pk_m_KC);
  x[PK_z_KC][id] = trap(DT, pk_z_KC_inf(Ca_val), 10.0, x[PK_z_KC][id]);
  G(PK_m_K2, pk_m_K2);
  x[PK_z_K2][id] = trap(DT, pk_z_K2_inf(Ca_val), 10.0, x[PK_z_K2][id]);
#undef G
  s->v[id] = vnew;
}

/* io_update_ion_RKC (io_ion.cu:91-126) */
static void io_ion_one(orc_sys *s, int id, double vnew, double DT) {
  double **x = s->ion;
  int lc = (int)s->compart[id];
  double v_old = s->v[id];
  double v_val = 0.5 * (vnew + v_old);
  double Ca_val = s->ca[id];
  double I = s->cond[IO_g_CaH][id] * x[IO_r][id] * x[IO_r][id] * (v_old - V_Ca_IO);
  double k1 = DT * (-I * CA_PH_IO - BETA_CA_IO * (Ca_val));
  double k2 = DT * (-I * CA_PH_IO - BETA_CA_IO * (Ca_val + k1 / 2.0));
  double k3 = DT * (-I * CA_PH_IO - BETA_CA_IO * (Ca_val + k2 / 2.0));
  double k4 = DT * (-I * CA_PH_IO - BETA_CA_IO * (Ca_val + k3));
  s->ca[id] += (k1 + k2 * 2.0 + k3 * 2.0 + k4) / 6.0;
  Ca_val = (Ca_val + s->ca[id]) / 2.0;
  x[IO_k][id] = trap(DT, io_k_inf(v_val), 1.0, x[IO_k][id]);
  x[IO_l][id] = trap(DT, io_l_inf(v_val), io_l_tau(v_val), x[IO_l][id]);
  x[IO_n][id] = trap(DT, io_n_inf(v_val), io_n_tau(v_val), x[IO_n][id]);
  x[IO_p][id] = trap(DT, io_p_inf(v_val), io_n_tau(v_val), x[IO_p][id]);
  x[IO_x][id] = trap(DT, io_x_inf(v_val), io_x_tau(v_val), x[IO_x][id]);
  x[IO_r][id] = trap(DT, io_r_inf(v_val), io_r_tau(v_val), x[IO_r][id]);
  x[IO_q][id] = trap(DT, io_q_inf(v_val), io_q_tau(v_val), x[IO_q][id]);
  x[IO_s][id] = trap(DT, io_s_inf(Ca_val), io_s_tau(Ca_val), x[IO_s][id]);
  x[IO_m][id] = io_m_inf(v_val);
  x[IO_h][id] = trap(DT, io_h_inf(v_val, lc), io_h_tau(v_val, lc), x[IO_h][id]);
  s->v[id] = vnew;
}

/* gr_update_ion_RKC_exp_imp (gr_ion.cu:461-480); Ca is never advanced */
static void gr_ion_one(orc_sys *s, int id, double vnew, double DT) {
  double **x = s->ion;
  double v_val = (s->v[id] + vnew) / 2.0;
  double Ca_val = s->ca[id];
  x[GR_n_KV][id] = trap(DT, gr_nKV_inf(v_val), gr_nKV_tau(v_val), x[GR_n_KV][id]);
  x[GR_a_KA][id] = trap(DT, gr_aKA_inf(v_val), gr_aKA_tau(v_val), x[GR_a_KA][id]);
  x[GR_b_KA][id] = trap(DT, gr_bKA_inf(v_val), gr_bKA_tau(v_val), x[GR_b_KA][id]);
  x[GR_ir_KIR][id] = trap(DT, gr_ir_inf(v_val), gr_ir_tau(v_val), x[GR_ir_KIR][id]);
  x[GR_s_KM][id] = trap(DT, gr_sKM_inf(v_val), gr_sKM_tau(v_val), x[GR_s_KM][id]);
  x[GR_c_KCa][id] = trap(DT, gr_cKCa_inf(v_val, Ca_val), gr_cKCa_tau(v_val, Ca_val), x[GR_c_KCa][id]);
  s->v[id] = vnew;
}

/* go_update_ion_RKC_exp_imp (go_ion.cu:379-437) */
static void go_ion_one(orc_sys *s, int id, double vnew, double DT) {
  double **x = s->ion;
  double v_old = s->v[id];
  double v_val = (v_old + vnew) / 2.0;
  double Ca_val = s->ca[id];
  double Ca2_val = s->ca2[id];
  double I1 = 1e-3 * s->cond[GO_g_CaHVA][id] / s->area[id] * x[GO_ch][id] * x[GO_ch][id] *
              x[GO_ci][id] * (v_old - V_Ca_GO);
  double I2 = 1e-3 * s->cond[GO_g_CaLVA][id] / s->area[id] * x[GO_cl][id] * x[GO_cl][id] *
              x[GO_cm][id] * (v_old - (s->rev_ca2[id]));
  double k1 = DT * (-I1 / (2.0 * F_GO * SHELL1_D_GO) - B_Ca1_GO * (Ca_val - Ca1_0_GO));
  double k2 = DT * (-I1 / (2.0 * F_GO * SHELL1_D_GO) - B_Ca1_GO * (Ca_val + k1 / 2.0 - Ca1_0_GO));
  double k3 = DT * (-I1 / (2.0 * F_GO * SHELL1_D_GO) - B_Ca1_GO * (Ca_val + k2 / 2.0 - Ca1_0_GO));
  double k4 = DT * (-I1 / (2.0 * F_GO * SHELL1_D_GO) - B_Ca1_GO * (Ca_val + k3 - Ca1_0_GO));
  s->ca[id] += (k1 + k2 * 2.0 + k3 * 2.0 + k4) / 6.0;
  k1 = DT * (-I2 / (2.0 * F_GO * SHELL1_D_GO) - B_Ca1_GO * (Ca2_val - Ca1_0_GO));
  k2 = DT * (-I2 / (2.0 * F_GO * SHELL1_D_GO) - B_Ca1_GO * (Ca2_val + k1 / 2.0 - Ca1_0_GO));
  k3 = DT * (-I2 / (2.0 * F_GO * SHELL1_D_GO) - B_Ca1_GO * (Ca2_val + k2 / 2.0 - Ca1_0_GO));
  k4 = DT * (-I2 / (2.0 * F_GO * SHELL1_D_GO) - B_Ca1_GO * (Ca2_val + k3 - Ca1_0_GO));
  s->ca2[id] += (k1 + k2 * 2.0 + k3 * 2.0 + k4) / 6.0;
  s->rev_ca2[id] = (1e3) * (8.313424 * (23.0 + 273.15)) / (2 * F_GO) * LOG(Ca1OUT_GO / s->ca2[id]);
  Ca_val = (Ca_val + s->ca[id]) / 2.0;
#define G(k, name) x[k][id] = trap(DT, name##_inf(v_val), name##_tau(v_val), x[k][id])
  G(GO_m_NaT, go_m_NaT); G(GO_h_NaT, go_h_NaT); G(GO_r_NaR, go_r_NaR);
  G(GO_s_NaR, go_s_NaR); G(GO_p_NaP, go_p_NaP); G(GO_n_KV, go_n_KV);
  G(GO_a_KA, go_a_KA); G(GO_b_KA, go_b_KA); G(GO_sl, go_sl);
  x[GO_c_KC][id] = trap(DT, go_c_KC_inf(v_val, Ca_val), go_c_KC_tau(v_val, Ca_val), x[GO_c_KC][id]);
  G(GO_ch, go_ch); G(GO_ci, go_ci); G(GO_cl, go_cl); G(GO_cm, go_cm);
  G(GO_hf1, go_hf1); G(GO_hf2, go_hf2); G(GO_hs1, go_hs1); G(GO_hs2, go_hs2);
#undef G
  s->v[id] = vnew;
}

/* *_update_ion_and_matrix minus b (solve_rkc.cu:1100-1117,1169-1185,1230-1251,1299-1317) */
void orc_ion_update(orc_sys *s, const double *vy, double DT) {
  int nc = s->nc;
  g_canon = s->canon;
  switch (s->type) {
    case ORC_GR:
      /* gr_Na_update_2order runs first, with elem[v] still the old V */
      for (int i = 0; i < nc; i++) gr_na_update(s, i, vy[i], s->v[i], DT);
      for (int i = 0; i < nc; i++) gr_ion_one(s, i, vy[i], DT);
      break;
    case ORC_GO:
      for (int i = 0; i < nc; i++) go_ion_one(s, i, vy[i], DT);
      for (int i = 0; i < nc; i++) go_kahp_update(s, i, DT);
      break;
    case ORC_PKJ:
      for (int i = 0; i < nc; i++) pkj_ion_one(s, i, vy[i], DT);
      break;
    case ORC_IO:
      for (int i = 0; i < nc; i++) io_ion_one(s, i, vy[i], DT);
      break;
  }
}

/* *_update_matrix (solve_rkc.cu:227-250, 289-312, 370-398, 413-435) */
void orc_update_b(orc_sys *s, const double *vy) {
  double **g = s->cond, **x = s->ion;
  g_canon = s->canon;
  for (int id = 0; id < s->nc; id++) {
    double lv = vy[id], r;
    switch (s->type) {
      case ORC_GR:
        r = (+g[GR_g_leak1][id] * (lv - V_LEAK1_GR) + g[GR_g_leak2][id] * (lv - V_LEAK2_GR) +
             g[GR_g_leak3][id] * (lv - V_LEAK3_GR) - s->iext[id] +
             +g[GR_g_Na][id] * (lv - V_Na_GR) * x[GR_o_Na][id] +
             g[GR_g_Ca][id] * (lv - V_Ca_GR) * x[GR_ch_Ca][id] * x[GR_ch_Ca][id] * x[GR_ci_Ca][id] +
             g[GR_g_KV][id] * (lv - V_K_GR) * x[GR_n_KV][id] * x[GR_n_KV][id] * x[GR_n_KV][id] * x[GR_n_KV][id] +
             g[GR_g_KIR][id] * (lv - V_K_GR) * x[GR_ir_KIR][id] +
             g[GR_g_KA][id] * (lv - V_K_GR) * x[GR_a_KA][id] * x[GR_a_KA][id] * x[GR_a_KA][id] * x[GR_b_KA][id] +
             g[GR_g_KCa][id] * (lv - V_K_GR) * x[GR_c_KCa][id] +
             g[GR_g_KM][id] * (lv - V_K_GR) * x[GR_s_KM][id]);
        break;
      case ORC_GO:
        r = (-s->iext[id] + g[GO_g_leak][id] * (lv - V_LEAK_GO) +
             g[GO_g_NaT][id] * (lv - V_Na_GO) * x[GO_m_NaT][id] * x[GO_m_NaT][id] * x[GO_m_NaT][id] * x[GO_h_NaT][id] +
             g[GO_g_NaR][id] * (lv - V_Na_GO) * x[GO_r_NaR][id] * x[GO_s_NaR][id] +
             g[GO_g_NaP][id] * (lv - V_Na_GO) * x[GO_p_NaP][id] +
             g[GO_g_CaHVA][id] * (lv - V_Ca_GO) * x[GO_ch][id] * x[GO_ch][id] * x[GO_ci][id] +
             g[GO_g_CaLVA][id] * (lv - s->rev_ca2[id]) * x[GO_cl][id] * x[GO_cl][id] * x[GO_cm][id] +
             g[GO_g_KAHP][id] * (lv - V_K_GO) * (x[GO_o1][id] + x[GO_o2][id]) +
             g[GO_g_KV][id] * (lv - V_K_GO) * x[GO_n_KV][id] * x[GO_n_KV][id] * x[GO_n_KV][id] * x[GO_n_KV][id] +
             g[GO_g_KA][id] * (lv - V_K_GO) * x[GO_a_KA][id] * x[GO_a_KA][id] * x[GO_a_KA][id] * x[GO_b_KA][id] +
             g[GO_g_KC][id] * (lv - V_K_GO) * x[GO_c_KC][id] +
             g[GO_g_Kslow][id] * (lv - V_K_GO) * x[GO_sl][id] +
             g[GO_g_HCN1][id] * (lv - V_H_GO) * (x[GO_hf1][id] + x[GO_hs1][id]) +
             g[GO_g_HCN2][id] * (lv - V_H_GO) * (x[GO_hf2][id] + x[GO_hs2][id]));
        break;
      case ORC_PKJ: {
        double vca = s->rev_ca2[id];
        r = (-s->iext[id] + g[PK_g_leak][id] * (lv - V_LEAK_PKJ) +
             g[PK_g_NaF][id] * x[PK_m_NaF][id] * x[PK_m_NaF][id] * x[PK_m_NaF][id] * x[PK_h_NaF][id] * (lv - V_Na_PKJ) +
             g[PK_g_NaP][id] * x[PK_m_NaP][id] * x[PK_m_NaP][id] * x[PK_m_NaP][id] * (lv - V_Na_PKJ) +
             g[PK_g_CaP][id] * x[PK_m_CaP][id] * x[PK_h_CaP][id] * (lv - vca) +
             g[PK_g_CaT][id] * x[PK_m_CaT][id] * x[PK_h_CaT][id] * (lv - vca) +
             g[PK_g_Kh][id] * x[PK_m_Kh1][id] * (lv - V_KH_PKJ) +
             g[PK_g_Kh][id] * x[PK_m_Kh2][id] * (lv - V_KH_PKJ) +
             g[PK_g_Kdr][id] * x[PK_m_Kdr][id] * x[PK_m_Kdr][id] * x[PK_h_Kdr][id] * (lv - V_K_PKJ) +
             g[PK_g_KM][id] * x[PK_m_KM][id] * (lv - V_K_PKJ) +
             g[PK_g_KA][id] * x[PK_m_KA][id] * x[PK_m_KA][id] * x[PK_m_KA][id] * x[PK_m_KA][id] * x[PK_h_KA][id] * (lv - V_K_PKJ) +
             g[PK_g_KC][id] * x[PK_m_KC][id] * x[PK_z_KC][id] * x[PK_z_KC][id] * (lv - V_K_PKJ) +
             g[PK_g_K2][id] * x[PK_m_K2][id] * x[PK_z_K2][id] * x[PK_z_K2][id] * (lv - V_K_PKJ));
        break;
      }
      default: /* IO */
        r = (-s->iext[id] + g[IO_g_leak][id] * (lv - V_LEAK_IO) +
             g[IO_g_CaL][id] * (lv - V_Ca_IO) * x[IO_k][id] * x[IO_k][id] * x[IO_k][id] * x[IO_l][id] +
             g[IO_g_Na][id] * (lv - V_Na_IO) * x[IO_m][id] * x[IO_m][id] * x[IO_m][id] * x[IO_h][id] +
             g[IO_g_Kdr][id] * (lv - V_K_IO) * x[IO_n][id] * x[IO_p][id] +
             g[IO_g_K][id] * (lv - V_K_IO) * x[IO_x][id] * x[IO_x][id] * x[IO_x][id] * x[IO_x][id] +
             g[IO_g_CaH][id] * (lv - V_Ca_IO) * x[IO_r][id] * x[IO_r][id] +
             g[IO_g_KCa][id] * (lv - V_K_IO) * x[IO_s][id] +
             g[IO_g_H][id] * (lv - V_H_IO) * x[IO_q][id]);
        break;
    }
    s->b[id] = r;
  }
}

/* io_gap_update + add_io_gap_val (gap.cu:141-160, solve_rkc.cu:401-410) */
static void io_gap_apply(orc_sys *s) {
  for (int e = 0; e < s->ngap; e++) {
    int pre = s->gap_pre[e], post = s->gap_post[e];
    double diff = (pre > -1) ? (s->v[post] - s->v[pre]) : 0.0;
    s->gap_cur[e] = s->gap_g[e] * (0.8 * EXP(-0.01 * diff * diff) + 0.2) * (diff);
  }
  for (int e = 0; e < s->ngap; e++) s->b[s->gap_post[e]] += s->gap_cur[e];
}

/* full *_update_ion_and_matrix */
static void ion_and_matrix(orc_sys *s, double sum_dt) {
  const double *vy = VEC(s, LY);
  orc_ion_update(s, vy, sum_dt);
  orc_update_b(s, vy);
  if (s->type == ORC_IO && s->ngap > 0) io_gap_apply(s);
  /* add_mfgr_val / add_gogr_val, go_update_matrix_new, pkj_update_matrix_new */
  if (s->syn_mode == 1) {
    for (int id = 0; id < s->nc; id++)
      for (int k = s->syn_row[id]; k < s->syn_row[id + 1]; k++) {
        int q = s->syn_idx[k];
        s->b[id] = s->b[id] + s->syn_val[q] * (vy[id] - s->syn_e[q]);
      }
  } else if (s->syn_mode == 2) {
    for (int id = 0; id < s->nc; id++) s->b[id] = s->b[id] + s->syn_buf[id];
  } else if (s->syn_mode == 3) {
    double decay = EXP(-sum_dt / 0.6);
    for (int id = 0; id < s->nc; id++) s->b[id] = s->b[id] + s->syn_buf[id] * decay;
  }
  s->n_ion++;
}

/* ------------------------------------------------------------------ */
/* setup: per-cell morphology -> elem/cond/CSR                          */
/* ------------------------------------------------------------------ */
/* dense-to-CSR with the diagonal kept explicit (pkj_solve.cu:152-183);
 * values are stored already sign-flipped for RKC (pkj_solve.cu:244-251):
 * off-diagonal +g, diagonal -(sum g).  mat is row-major ncomp*ncomp. */
typedef struct { int nnz; double *val; int *col, *row; } csr_t;

static csr_t dense_to_csr(const double *mat, int N) {
  csr_t c;
  int nnz = N;
  for (int i = 0; i < N * N; i++) nnz += (mat[i] > 0.0);
  c.nnz = nnz;
  c.val = zalloc(nnz); c.col = ialloc(nnz); c.row = ialloc(N + 1);
  int num = 0;
  for (int r = 0; r < N; r++) {
    int dig = -1;
    for (int cc = 0; cc < N; cc++) {
      double m = mat[r * N + cc];
      if (m > 0.0) { c.val[num] = -m; c.col[num] = cc; num++; }
      else if (r == cc) { c.val[num] = 0.0; c.col[num] = cc; dig = num; num++; }
    }
    for (int cc = 0; cc < N; cc++)
      if (cc != r) c.val[dig] += mat[r * N + cc];
    c.row[r + 1] = num;
  }
  return c;
}

static double rowf(const double *rows, int nf, int i, int f) { return rows[i * nf + f]; }

static void alloc_state(orc_sys *s) {
  int nc = s->nc;
  s->v = zalloc(nc); s->ca = zalloc(nc); s->cm = zalloc(nc); s->area = zalloc(nc);
  s->compart = zalloc(nc); s->iext = zalloc(nc);
  for (int k = 0; k < s->ncond; k++) s->cond[k] = zalloc(nc);
  for (int k = 0; k < s->nion; k++) s->ion[k] = zalloc(nc);
  s->ca2 = zalloc(nc); s->rev_ca2 = zalloc(nc); s->ca_old = zalloc(nc); s->shell = zalloc(nc);
  s->rev_fixed = ialloc(nc);
  s->b = zalloc(nc);
  for (int k = 0; k < NLOG; k++) { s->phys[k] = zalloc(nc); s->map[k] = k; }
  s->ede = zalloc(nc); s->vnew = zalloc(nc); s->dammy = zalloc(nc);
}

/* per-cell axial matrix for tree types (gr_solve.cu:37-43 and siblings) */
static void tree_mat(double *mat, int N, const int *parent, const double *rad,
                     const double *len, const double *Ra) {
  for (int i = 0; i < N * N; i++) mat[i] = 0.0;
  for (int i = 0; i < N; i++) {
    int d = parent[i];
    if (d >= 0) {
      mat[d + N * i] = (2.0 / ((Ra[i] * len[i]) / (rad[i] * rad[i] * M_PI) +
                               (Ra[d] * len[d]) / (rad[d] * rad[d] * M_PI)));
      mat[i + N * d] = mat[d + N * i];
    }
  }
}

/* insert one extra off-diagonal entry (row pre, column post, value g)
 * keeping each row sorted by column (pkj_solve.cu:4-26, go_solve.cu:163-196) */
static void csr_insert(orc_sys *s, int pre, int post, double g) {
  int pos = s->row[pre + 1];
  for (int j = s->row[pre]; j < s->row[pre + 1]; j++) {
    if (s->col[j] == post) { fprintf(stderr, "oracle: duplicate GJ %d->%d\n", pre, post); exit(1); }
    if (s->col[j] > post) { pos = j; break; }
  }
  int used = s->row[s->nc];
  for (int j = used; j > pos; j--) { s->col[j] = s->col[j - 1]; s->val[j] = s->val[j - 1]; }
  s->col[pos] = post;
  s->val[pos] = g;
  for (int i = pre + 1; i <= s->nc; i++) s->row[i]++;
}

static void replicate_csr(orc_sys *s, const csr_t *c, int extra) {
  int n = s->n, N = s->ncomp;
  s->nnz = c->nnz * n + extra;
  s->val = zalloc(s->nnz); s->col = ialloc(s->nnz); s->row = ialloc(s->nc + 1);
  for (int i = 0; i < n; i++) {
    for (int j = 0; j < c->nnz; j++) {
      s->val[j + c->nnz * i] = -c->val[j]; /* RKC sign flip */
      s->col[j + c->nnz * i] = c->col[j] + N * i;
    }
    for (int j = 0; j < N; j++) s->row[j + N * i] = c->row[j] + c->nnz * i;
  }
  s->row[s->nc] = c->nnz * n;
}

static int setup_cells(orc_sys *s, const orc_desc *d) {
  int N = s->ncomp, nf = orc_row_fields(s->type);
  const double *R = d->rows;
  double *rad = zalloc(N), *len = zalloc(N), *Ra = zalloc(N);
  int *parent = ialloc(N);
  double *mat = zalloc((size_t)N * N);
  /* template cell 0; conductances scale with area (gr.cu:41-55 etc.) */
  for (int i = 0; i < N; i++) {
    int i1 = (int)rowf(R, nf, i, 0);
    if (i1 != i) { fprintf(stderr, "oracle: rows must be in index order\n"); return -1; }
    parent[i] = (int)rowf(R, nf, i, 1);
    switch (s->type) {
      case ORC_GR: case ORC_GO: {
        double d1 = rowf(R, nf, i, 2), d2 = rowf(R, nf, i, 3), d3 = rowf(R, nf, i, 4), d4 = rowf(R, nf, i, 5);
        int i3 = (int)rowf(R, nf, i, 6);
        rad[i] = 0.5 * d1 * 1e-4; len[i] = d2 * 1e-4; Ra[i] = d3 * 1e-3;
        s->compart[i] = i3;
        s->area[i] = 2.0 * M_PI * rad[i] * len[i];
        double a = s->area[i];
        s->cm[i] = d4 * a;
        for (int k = 0; k < s->ncond; k++) s->cond[k][i] = rowf(R, nf, i, 7 + k) * a;
        break;
      }
      case ORC_PKJ: {
        double x = rowf(R, nf, i, 2), y = rowf(R, nf, i, 3), z = rowf(R, nf, i, 4), dd = rowf(R, nf, i, 5);
        int i3 = (int)rowf(R, nf, i, 6);
        double a;
        rad[i] = 0.5 * dd * 1e-4;
        Ra[i] = PKJ_RI;
        s->compart[i] = i3;
        static const double Gs[4][10] = {
            /* NaF NaP CaP CaT KH KDR KM KA KC K2   (pkj.cuh:29-65) */
            {7500.0, 1.0, 0.0, 0.5, 0.3, 600.0, 0.040, 15.0, 0.0, 0.0},
            {0.0, 0.0, 4.5, 0.5, 0.0, 60.0, 0.01, 2.0, 80.0, 0.39},
            {0.0, 0.0, 4.5, 0.5, 0.0, 0.0, 0.013, 0.0, 80.0, 0.39},
            {0.0, 0.0, 4.5, 0.5, 0.0, 0.0, 0.013, 0.0, 80.0, 0.39}};
        if (i3 == 0) {
          len[i] = dd * 1e-4;
          s->area[i] = 4.0 * M_PI * rad[i] * rad[i];
          a = s->area[i];
          s->cm[i] = PKJ_CM * a;
          s->shell[i] = (PKJ_SHELLD - 2 * pow(PKJ_SHELLD, 2) / (dd * 1e-4) +
                         4 * pow(PKJ_SHELLD, 3) / (3 * pow(dd * 1e-4, 2))) * s->area[i];
          s->cond[PK_g_leak][i] = 1.0 / PKJ_RM_S * a;
        } else {
          len[i] = sqrt(pow(x, 2) + pow(y, 2) + pow(z, 2)) * 1e-4;
          s->area[i] = 2.0 * M_PI * rad[i] * len[i];
          a = s->area[i];
          s->shell[i] = (PKJ_SHELLD - pow(PKJ_SHELLD, 2) / (dd * 1e-4)) * s->area[i];
          if (i3 == 3) {
            double other = a + len[i] * PKJ_SPINE_AREA * PKJ_SPINE_DENS;
            s->cm[i] = PKJ_CM * other;
            s->cond[PK_g_leak][i] = 1.0 / PKJ_RM_D * other;
          } else {
            s->cm[i] = PKJ_CM * a;
            s->cond[PK_g_leak][i] = 1.0 / PKJ_RM_D * a;
          }
        }
        for (int k = 0; k < 10; k++) s->cond[1 + k][i] = Gs[i3][k] * a;
        break;
      }
      case ORC_IO: {
        double d1 = rowf(R, nf, i, 2), d2 = rowf(R, nf, i, 3), d4 = rowf(R, nf, i, 4);
        int i3 = (int)rowf(R, nf, i, 5);
        rad[i] = 0.5 * d1 * 1e-4; len[i] = d2 * 1e-4;
        s->compart[i] = i3;
        s->area[i] = 2.0 * M_PI * rad[i] * len[i];
        s->cm[i] = d4;
        /* io.cu:48-82 */
        static const double Gio[3][8] = {
            {0.016 / (1 * 1.0), 0.0, 0.0, 0.0, 0.0, 4.5 / (1 * 1.0), 35.0 / (1 * 1.0), 0.15 / (1 * 1.0)},
            {0.016, 0.83, 120.0, 9.0, 5.0, 0.0, 0.0, 0.0},
            {0.016, 0.0, 240.0, 0.0, 20.0, 0.0, 0.0, 0.0}};
        for (int k = 0; k < 8; k++) s->cond[k][i] = Gio[i3][k];
        break;
      }
    }
  }
  /* axial matrix */
  if (s->type == ORC_IO) {
    /* io_solve.cu:37-65: asymmetric dendrite/soma/axon coupling */
    for (int i = 0; i < N * N; i++) mat[i] = 0.0;
    for (int i = 0; i < N; i++) {
      int dd = parent[i], i3 = (int)s->compart[i];
      double lg = 0.0, lgr = 0.0;
      if (dd >= 0) {
        if (i3 == 0 && dd == 1) { lg = (G_INT_IO / (1.0 - G_P_DS_IO)); lgr = (G_INT_IO / (G_P_DS_IO)); }
        else if (i3 == 1 && dd == 2) { lg = (G_INT_IO / (G_P_SA_IO)); lgr = (G_INT_IO / (1.0 - G_P_SA_IO)); }
        else if (i3 == 0 && dd < 1) { lg = lgr = (G_INT_IO / (0.5)); }
        mat[dd + N * i] = lg;
        mat[i + N * dd] = lgr;
      }
    }
  } else {
    tree_mat(mat, N, parent, rad, len, Ra);
  }
  csr_t c = dense_to_csr(mat, N);

  /* replicate cell 0 to all cells */
  for (int ci = 1; ci < s->n; ci++)
    for (int j = 0; j < N; j++) {
      int g = j + N * ci;
      s->compart[g] = s->compart[j]; s->cm[g] = s->cm[j]; s->area[g] = s->area[j];
      s->shell[g] = s->shell[j];
      for (int k = 0; k < s->ncond; k++) s->cond[k][g] = s->cond[k][j];
    }

  /* gap junctions written into the CSR (GO: go_solve.cu:51-81,160-196;
   * PKJ: pkj_solve.cu:79-120,200-236) */
  int n_gj = 0;
  int *gpre = NULL, *gpost = NULL;
  double ggj = 0.0;
  if (s->type == ORC_GO && d->go_gj && s->n > 1) {
    int gx = s->nx, gy = s->ny;
    n_gj = 2 * ((gx - 1) * gy + (gy - 1) * gx);
    gpre = ialloc(n_gj); gpost = ialloc(n_gj);
    int c_gj = 0;
    for (int y = 0; y < gy; y++)
      for (int x = 0; x < gx - 1; x++) {
        gpre[c_gj * 2] = (y * gx + x) * N; gpre[c_gj * 2 + 1] = (y * gx + x + 1) * N; c_gj++;
      }
    for (int x = 0; x < gx; x++)
      for (int y = 0; y < gy - 1; y++) {
        gpre[c_gj * 2] = (y * gx + x) * N; gpre[c_gj * 2 + 1] = ((y + 1) * gx + x) * N; c_gj++;
      }
    for (int i = 0; i < n_gj; i += 2) { gpost[i + 1] = gpre[i]; gpost[i] = gpre[i + 1]; }
    ggj = G_GJ_GO;
  }
  if (s->type == ORC_PKJ && d->pkj_gj && s->n > 1 && d->n_gj_pairs > 0) {
    int px = s->nx, py = s->ny, G = d->n_gj_pairs;
    n_gj = 2 * G * (px - 1) * py;
    gpre = ialloc(n_gj); gpost = ialloc(n_gj);
    int c_gj = 0;
    for (int y = 0; y < py; y++)
      for (int x = 0; x < px - 1; x++)
        for (int i = 0; i < G; i++) {
          gpre[c_gj * 2] = d->gj_pairs[2 * i] + (x + y * px) * N;
          gpre[c_gj * 2 + 1] = d->gj_pairs[2 * i + 1] + ((x + 1) + y * px) * N;
          c_gj++;
        }
    for (int i = 0; i < n_gj; i += 2) { gpost[i + 1] = gpre[i]; gpost[i] = gpre[i + 1]; }
    ggj = G_GJ_PKJ;
  }
  replicate_csr(s, &c, n_gj);
  for (int i = 0; i < n_gj; i++) {
    /* the diagonal gains the GJ conductance (sign-flipped storage) */
    int pre = gpre[i];
    for (int j = s->row[pre]; j < s->row[pre + 1]; j++)
      if (s->col[j] == pre) { s->val[j] -= ggj; break; }
    csr_insert(s, pre, gpost[i], ggj);
  }
  free(gpre); free(gpost);
  free(c.val); free(c.col); free(c.row);
  free(rad); free(len); free(Ra); free(parent); free(mat);
  return 0;
}

/* per-type initial state (*_initialize_ion: gr_ion.cu:635-672,
 * go_ion.cu:590-634, pkj_ion.cu:360-395, io_ion.cu:163-194) */
static void init_state(orc_sys *s, const double *jit) {
  int N = s->ncomp;
  for (int i = 0; i < s->nc; i++) {
    double r = jit[i / N];
    double **x = s->ion;
    switch (s->type) {
      case ORC_PKJ: {
        s->v[i] = V_INIT_PKJ + 2.0 * r;
        s->ca[i] = Ca1_0_PKJ;
        s->rev_ca2[i] = V_Ca_PKJ;
        s->iext[i] = 0.0;
        double v = s->v[i], ca = s->ca[i];
        x[PK_m_NaF][i] = pk_m_NaF_inf(v); x[PK_h_NaF][i] = pk_h_NaF_inf(v);
        x[PK_m_NaP][i] = pk_m_NaP_inf(v); x[PK_m_CaP][i] = pk_m_CaP_inf(v);
        x[PK_h_CaP][i] = pk_h_CaP_inf(v); x[PK_m_CaT][i] = pk_m_CaT_inf(v);
        x[PK_h_CaT][i] = pk_h_CaT_inf(v); x[PK_m_Kh1][i] = pk_m_Kh1_inf(v);
        x[PK_m_Kh2][i] = pk_m_Kh2_inf(v); x[PK_m_Kdr][i] = pk_m_Kdr_inf(v);
        x[PK_h_Kdr][i] = pk_h_Kdr_inf(v); x[PK_m_KM][i] = pk_m_KM_inf(v);
        x[PK_m_KA][i] = pk_m_KA_inf(v); x[PK_h_KA][i] = pk_h_KA_inf(v);
        x[PK_m_KC][i] = pk_m_KC_inf(v); x[PK_z_KC][i] = pk_z_KC_inf(ca);
        x[PK_m_K2][i] = pk_m_K2_inf(v); x[PK_z_K2][i] = pk_z_K2_inf(ca);
        s->rev_fixed[i] = (i % 1599 == 0);
        break;
      }
      case ORC_IO: {
        s->v[i] = V_INIT_IO + 10.0 * r;
        s->iext[i] = 0.0;
        double v = s->v[i];
        int lc = (int)s->compart[i];
        x[IO_k][i] = io_k_inf(v); x[IO_l][i] = io_l_inf(v); x[IO_n][i] = io_n_inf(v);
        x[IO_p][i] = io_p_inf(v); x[IO_x][i] = io_x_inf(v); x[IO_r][i] = io_r_inf(v);
        x[IO_q][i] = io_q_inf(v);
        double I = s->cond[IO_g_CaH][i] * x[IO_r][i] * x[IO_r][i] * (v - V_Ca_IO);
        s->ca[i] = -I * CA_PH_IO / BETA_CA_IO;
        x[IO_s][i] = io_s_inf(s->ca[i]);
        x[IO_m][i] = io_m_inf(v);
        x[IO_h][i] = io_h_inf(v, lc);
        break;
      }
      case ORC_GR: {
        s->v[i] = V_INIT_GR + 2.0 * r;
        s->ca[i] = Ca1_0_GR;
        s->iext[i] = 0.0;
        double v = s->v[i], ca = s->ca[i];
        x[GR_n_KV][i] = gr_nKV_inf(v); x[GR_a_KA][i] = gr_aKA_inf(v);
        x[GR_b_KA][i] = gr_bKA_inf(v); x[GR_ir_KIR][i] = gr_ir_inf(v);
        x[GR_s_KM][i] = gr_sKM_inf(v); x[GR_c_KCa][i] = gr_cKCa_inf(v, ca);
        x[GR_ch_Ca][i] = gr_ch_inf(v); x[GR_ci_Ca][i] = gr_ci_inf(v);
        for (int k = GR_o_Na; k <= GR_i6; k++) x[k][i] = 0.0;
        x[GR_c1][i] = 1.0;
        break;
      }
      case ORC_GO: {
        s->v[i] = V_INIT_GO + 2.0 * r;
        s->ca[i] = Ca1_0_GO; s->ca2[i] = Ca1_0_GO; s->rev_ca2[i] = V_Ca_GO;
        s->ca_old[i] = Ca1_0_GO;
        s->iext[i] = 0.0;
        double v = s->v[i], ca = s->ca[i];
        x[GO_m_NaT][i] = go_m_NaT_inf(v); x[GO_h_NaT][i] = go_h_NaT_inf(v);
        x[GO_r_NaR][i] = go_r_NaR_inf(v); x[GO_s_NaR][i] = go_s_NaR_inf(v);
        x[GO_p_NaP][i] = go_p_NaP_inf(v); x[GO_n_KV][i] = go_n_KV_inf(v);
        x[GO_a_KA][i] = go_a_KA_inf(v); x[GO_b_KA][i] = go_b_KA_inf(v);
        x[GO_c_KC][i] = go_c_KC_inf(v, ca); x[GO_sl][i] = go_sl_inf(v);
        x[GO_ch][i] = go_ch_inf(v); x[GO_ci][i] = go_ci_inf(v);
        x[GO_cl][i] = go_cl_inf(v); x[GO_cm][i] = go_cm_inf(v);
        x[GO_hf1][i] = go_hf1_inf(v); x[GO_hf2][i] = go_hf2_inf(v);
        x[GO_hs1][i] = go_hs1_inf(v); x[GO_hs2][i] = go_hs2_inf(v);
        x[GO_o1][i] = 0.0; x[GO_o2][i] = 0.0; x[GO_c2][i] = 0.0; x[GO_c3][i] = 0.0;
        x[GO_c4][i] = 0.0; x[GO_c1][i] = 1.0;
        break;
      }
    }
  }
}

/* IO gap network (gap.cu:4-120), including the idy = id / ny indexing */
static void io_gap_build(orc_sys *s, const orc_desc *d) {
  int nx = s->nx, ny = s->ny, n = s->n;
  s->ngap = 4 * n;
  s->gap_pre = ialloc(s->ngap); s->gap_post = ialloc(s->ngap);
  s->gap_cur = zalloc(s->ngap); s->gap_g = zalloc(s->ngap);
  for (int id = 0; id < n; id++) {
    int idx = id % nx, idy = id / ny;
    int L = id - 1, U = id - nx, Rr = id + 1, D = id + nx;
    /* the reference's else-if chain, in its order (first match wins) */
    if (idx == 0 && idy == 0) { L = -1; U = -1; }
    else if (idx == nx - 1 && idy == 0) { U = -1; Rr = -1; }
    else if (idx == 0 && idy == ny - 1) { L = -1; D = -1; }
    else if (idx == nx - 1 && idy == ny - 1) { Rr = -1; D = -1; }
    else if (idy == 0) { U = -1; }
    else if (idy == ny - 1) { D = -1; }
    else if (idx == 0) { L = -1; }
    else if (idx == nx - 1) { Rr = -1; }
    int nb[4] = {L, U, Rr, D};
    for (int k = 0; k < 4; k++) {
      s->gap_post[id * 4 + k] = id * 3;
      s->gap_pre[id * 4 + k] = nb[k] * 3; /* -1 becomes -3: "no neighbour" */
      s->gap_g[id * 4 + k] = d->io_gap_g ? d->io_gap_g[id * 4 + k] : G_C_IO;
    }
  }
}

int orc_nc(const orc_sys *s) { return s->nc; }
int orc_n(const orc_sys *s) { return s->n; }

orc_sys *orc_create(const orc_desc *d) {
  orc_sys *s = (orc_sys *)calloc(1, sizeof(orc_sys));
  s->type = d->type; s->nx = d->nx; s->ny = d->ny; s->n = d->nx * d->ny;
  s->ncomp = d->ncomp; s->nc = s->n * s->ncomp;
  switch (s->type) {
    case ORC_GR: s->ncond = GR_NCOND; s->nion = GR_NION; break;
    case ORC_GO: s->ncond = GO_NCOND; s->nion = GO_NION; break;
    case ORC_PKJ: s->ncond = PK_NCOND; s->nion = PK_NION; break;
    default: s->ncond = IO_NCOND; s->nion = IO_NION; break;
  }
  alloc_state(s);
  if (setup_cells(s, d) != 0) { orc_destroy(s); return NULL; }
  if (d->cond_scale_ch)
    for (int i = 0; i < s->nc; i++)
      for (int k = 0; k < s->ncond; k++)
        s->cond[k][i] = s->cond[k][i] * d->cond_scale_ch[(size_t)(i / s->ncomp) * s->ncond + k];
  else if (d->cond_scale)
    for (int i = 0; i < s->nc; i++)
      for (int k = 0; k < s->ncond; k++) s->cond[k][i] = s->cond[k][i] * d->cond_scale[i / s->ncomp];
  /* the reference computes the initial gating on the host with libm
   * (*_initialize_ion), so both modes use the platform exp here */
  g_canon = 0;
  init_state(s, d->jitter);
  if (s->type == ORC_IO && d->io_gap && s->n > 1) io_gap_build(s, d);
  s->stim_comp = ialloc(s->n); s->stim_amp = zalloc(s->n);
  s->stim_t0 = zalloc(s->n); s->stim_t1 = zalloc(s->n);
  for (int c = 0; c < s->n; c++) {
    s->stim_comp[c] = d->stim_comp ? d->stim_comp[c] : -1;
    s->stim_amp[c] = d->stim_amp ? d->stim_amp[c] : 0.0;
    s->stim_t0[c] = d->stim_t0 ? d->stim_t0[c] : 0.0;
    s->stim_t1[c] = d->stim_t1 ? d->stim_t1[c] : 0.0;
  }
  static const double tol_def[4] = {1.0e-9, 1.0e-6, 1.0e-6, 1.0e-6};   /* solve_rkc.cuh:28-31 */
  const double hmin_def[4] = {pow(2.0, -12.0), pow(2.0, -10.0), pow(2.0, -10.0), pow(2.0, -10.0)};
  s->canon = d->canon;
  s->invcm = zalloc(s->nc);
  s->scratch = zalloc(s->nc);
  for (int i = 0; i < s->nc; i++) s->invcm[i] = 1.0 / s->cm[i];
  s->atol = s->rtol = (d->tol > 0) ? d->tol : tol_def[s->type];
  s->hmin = (d->hmin > 0) ? d->hmin : hmin_def[s->type];
  return s;
}

void orc_destroy(orc_sys *s) {
  if (!s) return;
  free(s->v); free(s->ca); free(s->cm); free(s->area); free(s->compart); free(s->iext);
  for (int k = 0; k < s->ncond; k++) free(s->cond[k]);
  for (int k = 0; k < s->nion; k++) free(s->ion[k]);
  free(s->ca2); free(s->rev_ca2); free(s->ca_old); free(s->shell); free(s->rev_fixed);
  free(s->val); free(s->col); free(s->row); free(s->b);
  for (int k = 0; k < NLOG; k++) free(s->phys[k]);
  free(s->ede); free(s->vnew); free(s->dammy);
  free(s->stim_comp); free(s->stim_amp); free(s->stim_t0); free(s->stim_t1);
  free(s->gap_pre); free(s->gap_post); free(s->gap_cur); free(s->gap_g);
  free(s->invcm); free(s->scratch);
  free(s->syn_row); free(s->syn_idx); free(s->syn_buf);
  free(s);
}

/* ------------------------------------------------------------------ */
/* RKC integrator (solve_rkc.cu:165-196, 438-1096)                     */
/* ------------------------------------------------------------------ */
/* dydt (solve_rkc.cu:178-196) */
static void dydt(orc_sys *s, const double *y, double *dy) {
  if (s->canon) {
    /* diagonal entries contribute val * (y_i - y_i) = 0 and are skipped */
    for (int i = 0; i < s->nc; i++) {
      double d = (-(s->b[i]));
      const double yi = y[i];
      for (int j = s->row[i]; j < s->row[i + 1]; j++) {
        if (s->col[j] == i) continue;
        d = fma(s->val[j], y[s->col[j]] - yi, d);
      }
      dy[i] = d * s->invcm[i];
    }
    return;
  }
  for (int i = 0; i < s->nc; i++) {
    double d = (-(s->b[i]));
    const double yi = y[i];
    for (int j = s->row[i]; j < s->row[i + 1]; j++) d += s->val[j] * (y[s->col[j]] - yi);
    dy[i] = d / s->cm[i];
  }
}

static double dot(const double *a, const double *b, int n) {
  double r = 0.0;
  for (int i = 0; i < n; i++) r += a[i] * b[i];
  return r;
}

/* sum of squares: sequential (reference mode) or the canonical tree */
static double sumsq(orc_sys *s, const double *a, int n) {
  if (!s->canon) return dot(a, a, n);
  for (int i = 0; i < n; i++) s->scratch[i] = a[i] * a[i];
  return tree_sum(s->scratch, n);
}

static double fmax_ori(double a, double b) { return (a > b) ? a : b; }

static int nint(double x) {
  if (x - (double)(int)x < 0.5) return (int)((double)(int)x);
  else return (int)((double)(int)(x + 0.9));
}

/* rkcrho (solve_rkc.cu:563-754): nonlinear power method for rho(J) */
static void rkcrho(orc_sys *s) {
  int nc = s->nc;
  const int itmax = 1000;
  double sprad_old[3] = {0.0, 0.0, 0.0};
  const double uround = UROUND, sqrtu = sqrt(UROUND), small = 1.0 / 0.125;
  double *yn = VEC(s, LYN), *fn = VEC(s, LFN), *v1 = VEC(s, LV1), *v2 = VEC(s, LV2);
  double *ede = s->ede, *dam = s->dammy;
  double ynrm = sqrt(sumsq(s, yn, nc));
  double vnrm = sqrt(sumsq(s, ede, nc));
  double dynrm, sigma, sigmal, dfnrm;
  s->n_rho++;
  if (ynrm != 0.0 && vnrm != 0.0) {
    dynrm = ynrm * sqrtu;
    double al = dynrm / vnrm;
    if (s->canon) for (int i = 0; i < nc; i++) v1[i] = fma(al, ede[i], yn[i]);
    else for (int i = 0; i < nc; i++) v1[i] = al * ede[i] + yn[i];
  } else if (ynrm != 0.0) {
    dynrm = ynrm * sqrtu;
    if (s->canon) for (int i = 0; i < nc; i++) v1[i] = fma(sqrtu, yn[i], yn[i]);
    else for (int i = 0; i < nc; i++) v1[i] = sqrtu * yn[i] + yn[i];
  } else if (vnrm != 0.0) {
    dynrm = uround;
    double al = dynrm / vnrm;
    for (int i = 0; i < nc; i++) v1[i] = al * ede[i];
  } else {
    dynrm = uround;
    for (int i = 0; i < nc; i++) v1[i] = dynrm;
  }
  sigma = 0.0;
  for (int iter = 0; iter < itmax; iter++) {
    s->n_rho_iter++;
    dydt(s, v1, v2);
    for (int i = 0; i < nc; i++) dam[i] = -1.0 * fn[i] + v2[i];
    dfnrm = sqrt(sumsq(s, dam, nc));
    sigmal = sigma;
    sigma = dfnrm / dynrm;
    sprad_old[0] = sprad_old[1];
    sprad_old[1] = sprad_old[2];
    sprad_old[2] = s->sprad;
    s->sprad = 1.2 * sigma;
    if (iter >= 1 && fabs(sigma - sigmal) <= fmax_ori(sigma, small) * 0.001) {
      for (int i = 0; i < nc; i++) ede[i] = -1.0 * yn[i] + v1[i];
      return;
    }
    if (iter > itmax / 2) {
      if ((fabs(sprad_old[2] - sprad_old[0]) < 0.00001) && (fabs(sprad_old[1] - s->sprad) < 0.00001)) {
        s->sprad = (s->sprad + sprad_old[2]) / 2.0;
        for (int i = 0; i < nc; i++) ede[i] = -1.0 * yn[i] + v1[i];
        return;
      }
    }
    if (dfnrm != 0.0) {
      double al = dynrm / dfnrm;
      if (s->canon) {
        for (int i = 0; i < nc; i++) v1[i] = fma(al, fn[i] - v2[i], yn[i]);
      } else {
        for (int i = 0; i < nc; i++) v1[i] = -1.0 * v2[i] + fn[i];
        for (int i = 0; i < nc; i++) v1[i] = al * v1[i] + yn[i];
      }
    } else {
      int idx = iter % nc;
      v1[idx] = 2.0 * yn[idx] - v1[idx];
    }
  }
  s->idid = 6;
}

/* set_initial_vec + rkcrho + set_initial_absh (solve_rkc.cu:438-560, 757-791) */
int orc_init(orc_sys *s) {
  int nc = s->nc;
  g_canon = s->canon;
  orc_update_b(s, s->v);
  for (int i = 0; i < nc; i++) {
    s->vnew[i] = s->v[i]; VEC(s, LY)[i] = s->v[i]; VEC(s, LYN)[i] = s->v[i];
    VEC(s, LFN)[i] = 0.0; s->ede[i] = 0.0; VEC(s, LV1)[i] = 0.0; VEC(s, LV2)[i] = 0.0;
  }
  memset(s->hw, 0, sizeof s->hw);
  s->mmax = s->absh = s->sprad = s->naccpt = s->idid = s->gt = s->gt_old = s->lt = 0.0;
  s->errold = s->hold = s->nstsig = 0.0;
  s->cbrt_errold = 0.0;
  s->hw[2] = nc; s->hw[3] = UROUND; s->hw[4] = sqrt(UROUND); s->hw[5] = H_MAX; s->hw[6] = s->hmin;
  s->tend = H_MAX;
  s->last = 1; s->newspc = 1; s->jacatt = 0;
  s->sum_dt = 0.0;
  s->integ = pow(2.0, log10(s->atol));
  dydt(s, VEC(s, LYN), VEC(s, LFN));
  memcpy(s->ede, VEC(s, LFN), sizeof(double) * nc);

  rkcrho(s);

  /* set_initial_absh */
  double *yn = VEC(s, LYN), *fn = VEC(s, LFN), *v1 = VEC(s, LV1), *v2 = VEC(s, LV2);
  double absh = H_MAX;
  if (s->sprad * absh > 1.0) absh = 1.0 / s->sprad;
  absh = fmax_ori(absh, s->hw[6]);
  if (s->canon) for (int i = 0; i < nc; i++) v1[i] = fma(absh, fn[i], yn[i]);
  else for (int i = 0; i < nc; i++) v1[i] = yn[i] + absh * fn[i];
  dydt(s, v1, v2);
  for (int i = 0; i < nc; i++) {
    double wt = s->canon ? fma(s->rtol, fabs(yn[i]), s->atol) : s->atol + s->rtol * fabs(yn[i]);
    if (wt == 0.0) { s->idid = 3.0; return 3; }
    s->dammy[i] = 1.0 / wt;
  }
  for (int i = 0; i < nc; i++) s->dammy[i] = (v2[i] - fn[i]) * s->dammy[i];
  double est = sumsq(s, s->dammy, nc);
  est = absh * sqrt(est / nc);
  if (0.1 * absh < H_MAX * sqrt(est)) absh = fmax_ori(0.1 * absh / sqrt(est), s->hw[6]);
  else absh = H_MAX;
  s->absh = absh;
  s->mmax = nint(sqrt(s->rtol / (10.0 * UROUND)));
  return (int)s->idid;
}

static void rot3_step_end(orc_sys *s) {
  /* step's final shuffle (solve_rkc.cu:902-905) */
  int t = s->map[LY];
  s->map[LY] = s->map[LV1]; s->map[LV1] = s->map[LV2]; s->map[LV2] = t;
}

/* step (solve_rkc.cu:816-906) */
static void step(orc_sys *s, double h, int m) {
  int nc = s->nc;
  double ajm1, arg, bj, bjm1, bjm2, dzj, dzjm1, dzjm2, d2zj, d2zjm1, d2zjm2, mu, mus, nu,
      temp1, temp2, w0, w1, zj, zjm1, zjm2;
  w0 = 1.0 + 2.0 / (13.0 * m * m);
  temp1 = w0 * w0 - 1.0;
  temp2 = sqrt(temp1);
  arg = m * log(w0 + temp2);
  w1 = sinh(arg) * temp1 / (cosh(arg) * m * temp2 - w0 * sinh(arg));
  bjm1 = 1.0 / ((2.0 * w0) * (2.0 * w0));
  bjm2 = bjm1;
  mus = w1 * bjm1;
  {
    double *yn = VEC(s, LYN), *fn = VEC(s, LFN), *v1 = VEC(s, LV1), *v2 = VEC(s, LV2);
    memcpy(v2, yn, sizeof(double) * nc);
    double hm = h * mus;
    if (s->canon) for (int i = 0; i < nc; i++) v1[i] = fma(hm, fn[i], yn[i]);
    else for (int i = 0; i < nc; i++) v1[i] = hm * fn[i] + yn[i];
  }
  zjm1 = w0; zjm2 = 1.0; dzjm1 = 1.0; dzjm2 = 0.0; d2zjm1 = 0.0; d2zjm2 = 0.0;
  for (int j = 1; j < m; j++) {
    zj = 2.0 * w0 * zjm1 - zjm2;
    dzj = 2.0 * w0 * dzjm1 - dzjm2 + 2.0 * zjm1;
    d2zj = 2.0 * w0 * d2zjm1 - d2zjm2 + 4.0 * dzjm1;
    bj = d2zj / (dzj * dzj);
    ajm1 = 1.0 - zjm1 * bjm1;
    mu = 2.0 * w0 * bj / bjm1;
    nu = -bj / bjm2;
    mus = mu * w1 / w0;
    double *y = VEC(s, LY), *yn = VEC(s, LYN), *fn = VEC(s, LFN), *v1 = VEC(s, LV1), *v2 = VEC(s, LV2);
    dydt(s, v1, y);
    double omn = (1.0 - mu - nu), hm = h * mus;
    if (s->canon) {
      for (int i = 0; i < nc; i++) {
        double t = mu * v1[i];
        t = fma(nu, v2[i], t);
        t = fma(omn, yn[i], t);
        double u = fma(-ajm1, fn[i], y[i]);
        y[i] = fma(hm, u, t);
      }
    } else {
      for (int i = 0; i < nc; i++)
        y[i] = mu * v1[i] + nu * v2[i] + omn * yn[i] + hm * (y[i] - ajm1 * fn[i]);
    }
    /* rotate v2 <- v1 <- y <- v2 (solve_rkc.cu:879-883) */
    int t = s->map[LV2];
    s->map[LV2] = s->map[LV1]; s->map[LV1] = s->map[LY]; s->map[LY] = t;
    bjm2 = bjm1; bjm1 = bj; zjm2 = zjm1; zjm1 = zj; dzjm2 = dzjm1; dzjm1 = dzj;
    d2zjm2 = d2zjm1; d2zjm1 = d2zj;
  }
  rot3_step_end(s);
  s->n_stage += m;
}

/* rkclow (solve_rkc.cu:909-1096): one accepted step (or the hmin floor) */
static void rkclow(orc_sys *s) {
  int nc = s->nc, m;
  double err, fac, h, temp1, temp2;
  const double hmax = H_MAX, hmin = s->hw[6];
  int loop_num = 0;
  for (;;) {
    loop_num++;
    if (loop_num > 1000) return;
    if (s->newspc) { rkcrho(s); s->jacatt = 1; }
    s->last = 0;
    if (1.1 * s->absh >= fabs(s->tend - s->lt)) { s->absh = fabs(s->tend - s->lt); s->last = 1; }
    m = 1 + (int)(sqrt(1.54 * s->absh * s->sprad + 1.0));
    if (m > s->mmax) {
      m = (int)s->mmax;
      s->absh = (m * m - 1) / (1.54 * s->sprad);
      s->last = 0;
    }
    h = 1.0 * s->absh;
    if (h <= hmin) h = hmin;
    step(s, h, m);
    s->n_steps++;
    double *y = VEC(s, LY), *yn = VEC(s, LYN), *fn = VEC(s, LFN), *v1 = VEC(s, LV1);
    dydt(s, y, v1);
    err = 0.0;
    if (s->canon) {
      for (int i = 0; i < nc; i++) {
        double wt = fma(s->rtol, fmax_ori(fabs(y[i]), fabs(yn[i])), s->atol);
        double est = fma(0.4 * h, fn[i] + v1[i], 0.8 * (yn[i] - y[i]));
        double q = est / wt;
        s->scratch[i] = q * q;
      }
      err = tree_sum(s->scratch, nc);
    } else {
      for (int i = 0; i < nc; i++) {
        double wt = s->atol + s->rtol * fmax_ori(fabs(y[i]), fabs(yn[i]));
        double est = 0.8 * (yn[i] - y[i]) + 0.4 * h * (fn[i] + v1[i]);
        err += (est / wt) * (est / wt);
      }
    }
    if (s->idid == 3.0) return;
    err = sqrt(err / (double)nc);
    if (err > 1.0) {
      /* canonical: the same cube root as the accept path (cm_cbrt) */
      s->absh = 0.8 * s->absh / (g_canon ? cm_cbrt(err) : pow(err, 1.0 / 3.0));
      s->n_rej++;
      if (s->absh < hmin) {
        s->idid = 4;
      } else {
        s->newspc = !s->jacatt;
        continue;
      }
    }
    s->naccpt += 1;
    s->lt += h;
    s->gt = s->lt;
    s->jacatt = 0;
    /* nstsig is read but never stored back (solve_rkc.cu:1024-1026), so the
     * every-25-steps refresh of rho never fires */
    int l_nstsig = ((int)(s->nstsig) + 1) % 25;
    s->newspc = 0;
    if (l_nstsig == 0) s->newspc = !s->jacatt;
    s->hw[0] = h;
    s->hw[1] = s->lt;
    {
      int tmp = s->map[LV2];
      s->map[LV2] = s->map[LFN]; s->map[LFN] = s->map[LV1]; s->map[LV1] = s->map[LYN];
      s->map[LYN] = s->map[LY]; s->map[LY] = tmp;
    }
    fac = 10.0;
    if (s->canon) {
      /* canonical: err^(1/3) once; err^(2/3) as its square; errold^(1/3)
       * carried over from the previous accepted step */
      const double cr = cm_cbrt(err);
      if (s->naccpt == 1) {
        temp2 = cr;
        if (0.8 < fac * temp2) fac = 0.8 / temp2;
      } else {
        temp1 = 0.8 * s->absh * s->cbrt_errold;
        temp2 = fabs(s->hold) * (cr * cr);
        if (temp1 < fac * temp2) fac = temp1 / temp2;
      }
      s->cbrt_errold = cr;
    } else if (s->naccpt == 1) {
      temp2 = POW(err, 1.0 / 3.0);
      if (0.8 < fac * temp2) fac = 0.8 / temp2;
    } else {
      temp1 = 0.8 * s->absh * POW(s->errold, 1.0 / 3.0);
      temp2 = fabs(s->hold) * POW(err, 2.0 / 3.0);
      if (temp1 < fac * temp2) fac = temp1 / temp2;
    }
    s->absh = fmax_ori(0.1, fac) * s->absh;
    s->absh = fmax_ori(hmin, fmin(hmax, s->absh));
    s->errold = err;
    s->hold = h;
    s->idid = s->last ? 1 : 2;
    return;
  }
}

/* rkcint (solve_rkc.cu:795-813) */
static void rkcint(orc_sys *s) {
  double hlast = s->hw[0], lt = s->hw[1], gtv = s->gt_old;
  double tlast = lt - hlast;
  double sv = (gtv - tlast) / hlast;
  double a1 = (1.0 + 2.0 * sv) * (sv - 1.0) * (sv - 1.0);
  double a2 = (3.0 - 2.0 * sv) * sv * sv;
  double b1 = hlast * sv * (sv - 1.0) * (sv - 1.0);
  double b2 = hlast * (sv - 1.0) * sv * sv;
  double *v1 = VEC(s, LV1), *v2 = VEC(s, LV2), *yn = VEC(s, LYN), *fn = VEC(s, LFN);
  if (s->canon)
    for (int i = 0; i < s->nc; i++)
      s->vnew[i] = fma(b2, fn[i], fma(b1, v2[i], fma(a2, yn[i], a1 * v1[i])));
  else
    for (int i = 0; i < s->nc; i++) s->vnew[i] = a1 * v1[i] + a2 * yn[i] + b1 * v2[i] + b2 * fn[i];
}

/* per-cell step current, evaluated at the start of each interval
 * (pkj_set_current pkj.cu:333-343 and siblings) */
static void set_current(orc_sys *s, double t) {
  for (int c = 0; c < s->n; c++) {
    int comp = s->stim_comp[c];
    if (comp < 0) continue;
    int g = comp + c * s->ncomp;
    s->iext[g] = 0;
    if (s->stim_t0[c] <= t && t < s->stim_t1[c]) s->iext[g] = s->stim_amp[c];
  }
}

/* *_solve_by_rkc (solve_rkc.cu:1122-1362) for one 0.125 ms interval */
int orc_advance(orc_sys *s, double t) {
  g_canon = s->canon;
  set_current(s, t);
  /* Golgi / Purkinje: synaptic current at interval start, before the pending
   * ion update (add_grgo_val_new 1199-1200, add_grpkj_val_new 1266-1269) */
  if (s->syn_mode == 2 || s->syn_mode == 3) {
    const double *vy = VEC(s, LY);
    for (int id = 0; id < s->nc; id++) {
      double acc = 0.0;
      for (int k = s->syn_row[id]; k < s->syn_row[id + 1]; k++) {
        int q = s->syn_idx[k];
        acc = acc + s->syn_val[q] * (vy[id] - s->syn_e[q]);
      }
      s->syn_buf[id] = acc;
    }
  }
  /* GR and IO compare with '>', GO and PKJ with '>=' (solve_rkc.cu:1148,1212,1284,1347) */
  const int ge = (s->type == ORC_GO || s->type == ORC_PKJ);
  if (s->sum_dt != 0.0) {
    ion_and_matrix(s, s->sum_dt);
    s->sum_dt = 0.0;
  }
  for (;;) {
    rkclow(s);
    s->sum_dt += s->gt - s->gt_old;
    s->gt_old = s->gt;
    int trig = ge ? (s->sum_dt >= s->integ) : (s->sum_dt > s->integ);
    if (trig && s->idid == 2.0) {
      ion_and_matrix(s, s->sum_dt);
      s->sum_dt = 0.0;
    }
    if (s->idid == 2.0) continue;
    else if (s->idid == 1.0) break;
    else return (int)s->idid;
  }
  rkcint(s);
  s->tend += H_MAX;
  return 0;
}

const double *orc_vnew(const orc_sys *s) { return s->vnew; }
const double *orc_elem_v(const orc_sys *s) { return s->v; }
const double *orc_b(const orc_sys *s) { return s->b; }
const double *orc_ion(const orc_sys *s, int k) { return (k >= 0 && k < s->nion) ? s->ion[k] : NULL; }
const double *orc_ca(const orc_sys *s) { return s->ca; }
const double *orc_cm(const orc_sys *s) { return s->cm; }
const double *orc_area(const orc_sys *s) { return s->area; }
const double *orc_cond(const orc_sys *s, int k) { return (k >= 0 && k < s->ncond) ? s->cond[k] : NULL; }
int orc_ncond(const orc_sys *s) { return s->ncond; }
int orc_nion(const orc_sys *s) { return s->nion; }
const double *orc_shell(const orc_sys *s) { return s->shell; }
const double *orc_rev_ca2(const orc_sys *s) { return s->rev_ca2; }
int orc_nnz(const orc_sys *s) { return s->row[s->nc]; }
const int *orc_row(const orc_sys *s) { return s->row; }
const int *orc_col(const orc_sys *s) { return s->col; }
const double *orc_val(const orc_sys *s) { return s->val; }
void orc_set_elem_v(orc_sys *s, const double *v) { memcpy(s->v, v, sizeof(double) * s->nc); }
void orc_set_ion(orc_sys *s, int k, const double *x) { memcpy(s->ion[k], x, sizeof(double) * s->nc); }
void orc_set_ca(orc_sys *s, const double *x) { memcpy(s->ca, x, sizeof(double) * s->nc); }

void orc_ctl(const orc_sys *s, double *o) {
  o[0] = s->absh; o[1] = s->sprad; o[2] = s->naccpt; o[3] = s->errold;
  o[4] = s->hold; o[5] = s->lt; o[6] = s->tend; o[7] = s->sum_dt;
}

void orc_stats(const orc_sys *s, long long *o) {
  o[0] = s->n_steps; o[1] = s->n_rej; o[2] = s->n_stage; o[3] = s->n_rho; o[4] = s->n_ion;
  o[5] = s->n_rho_iter;
}

void orc_draw_jitter(int type, int n, double *out) {
  for (int c = 0; c < n; c++) {
    if (type == ORC_GR || type == ORC_PKJ)
      out[c] = (((double)rand() + 1.0) / ((double)RAND_MAX + 2.0)) - 0.5;
    else
      out[c] = ((double)rand() / RAND_MAX) - 0.5;
  }
}

/* ------------------------------------------------------------------ */
/* network mode: systems plus the reference's chemical synapses         */
/* (syn.cu; main.cu:196-305 with network_sim true)                      */
/* ------------------------------------------------------------------ */
enum { SYN_MFGR, SYN_GRGO, SYN_GOGR, SYN_GRPKJ, SYN_KINDS };

struct orc_net {
  int nsys;
  orc_sys *sys[64];
  int n, cap;
  int *kind, *grp, *pre_sys, *pre_comp, *post_sys, *post_comp;
  double *w, *s0, *s1, *s2, *val, *old_v, *e;
  unsigned long long *ring; /* last 64 events per synapse, newest in bit 0 */
  int *delay;               /* intervals between an event and its effect */
  int ngrp;
  double rate[64][4];
  unsigned long long seed[64];
  double decay[8];
  long long interval;
};

orc_net *orc_net_create(void) {
  orc_net *n = (orc_net *)calloc(1, sizeof(orc_net));
  /* exp(-RKC_DT / tau), syn.cuh:14-15, 21-23, 32-33, 40 */
  static const double tau[8] = {1.2, 52.0, 1.5, 31.0, 170.0, 7.0, 59.0, 6.0};
  for (int k = 0; k < 8; k++) n->decay[k] = exp(-0.125 / tau[k]);
  return n;
}

int orc_net_add_system(orc_net *n, orc_sys *s) {
  if (n->nsys >= 64) return -1;
  n->sys[n->nsys] = s;
  return n->nsys++;
}

#define NET_GROW(f, T) n->f = (T *)realloc(n->f, (size_t)n->cap * sizeof(T))
int orc_net_add_synapses(orc_net *n, int kind, int count, const int *pre_sys, const int *pre_comp,
                         const int *post_sys, const int *post_comp, const double *w, double rate_base,
                         double rate_stim, double t0, double t1, unsigned long long seed) {
  /* E_MFGR, E_GRGO, E_GOGR, E_GRPKJ (syn.cuh:13,20,31,38) */
  static const double ekind[SYN_KINDS] = {0.0, 0.0, -82.0, 0.0};
  if (n->ngrp >= 64 || kind < 0 || kind >= SYN_KINDS) return -1;
  int g = n->ngrp++;
  int dflt = rate_base == 0.0 && rate_stim == 0.0 && t0 == 0.0 && t1 == 0.0;
  n->rate[g][0] = dflt ? 5.0 : rate_base;
  n->rate[g][1] = dflt ? 60.0 : rate_stim;
  n->rate[g][2] = dflt ? 900.0 : t0;
  n->rate[g][3] = dflt ? 1000.0 : t1;
  n->seed[g] = seed;
  if (n->n + count > n->cap) {
    n->cap = (n->n + count) * 2;
    NET_GROW(kind, int); NET_GROW(grp, int); NET_GROW(pre_sys, int); NET_GROW(pre_comp, int);
    NET_GROW(post_sys, int); NET_GROW(post_comp, int);
    NET_GROW(w, double); NET_GROW(s0, double); NET_GROW(s1, double); NET_GROW(s2, double);
    NET_GROW(val, double); NET_GROW(old_v, double); NET_GROW(e, double);
    NET_GROW(ring, unsigned long long); NET_GROW(delay, int);
  }
  int first = n->n;
  for (int i = 0; i < count; i++) {
    int k = n->n++;
    n->kind[k] = kind;
    n->grp[k] = g;
    n->pre_sys[k] = (kind == SYN_MFGR) ? -1 : pre_sys[i];
    n->pre_comp[k] = (kind == SYN_MFGR) ? 0 : pre_comp[i];
    n->post_sys[k] = post_sys[i];
    n->post_comp[k] = post_comp[i];
    n->w[k] = w[i];
    n->s0[k] = n->s1[k] = n->s2[k] = n->val[k] = 0.0;
    n->old_v[k] = 1000.0; /* syn.cu:176, 330, 510 */
    n->e[k] = ekind[kind];
    n->ring[k] = 0ull;
    n->delay[k] = 0;
  }
  return first;
}

/* CSR of each system's incoming synapses, ids in (kind, id) order */
int orc_net_build(orc_net *n) {
  for (int q = 0; q < n->nsys; q++) {
    orc_sys *s = n->sys[q];
    int cnt = 0;
    for (int k = 0; k < n->n; k++) cnt += (n->post_sys[k] == q);
    if (!cnt) continue;
    s->syn_row = ialloc((size_t)s->nc + 1);
    s->syn_idx = ialloc((size_t)cnt);
    s->syn_buf = zalloc((size_t)s->nc);
    for (int k = 0; k < n->n; k++)
      if (n->post_sys[k] == q) s->syn_row[n->post_comp[k] + 1]++;
    for (int c = 0; c < s->nc; c++) s->syn_row[c + 1] += s->syn_row[c];
    int *fill = ialloc((size_t)s->nc);
    for (int kd = 0; kd < SYN_KINDS; kd++)
      for (int k = 0; k < n->n; k++)
        if (n->post_sys[k] == q && n->kind[k] == kd) {
          int c = n->post_comp[k];
          s->syn_idx[s->syn_row[c] + fill[c]++] = k;
        }
    free(fill);
    s->syn_val = n->val;
    s->syn_e = n->e;
    s->syn_mode = (s->type == ORC_GR) ? 1 : (s->type == ORC_GO) ? 2 : (s->type == ORC_PKJ) ? 3 : 0;
    if (!s->syn_mode) return -1;
  }
  return 0;
}

/* SplitMix64 finaliser (Steele, Lea & Flood 2014) over (seed, synapse,
 * interval) -> (0, 1]: the Poisson draws, shared with the CUDA path */
static double syn_uniform(unsigned long long seed, long long id, long long interval) {
  unsigned long long z = seed ^ ((unsigned long long)id * 0xD1B54A32D192ED03ull) ^
                         ((unsigned long long)interval * 0x9E3779B97F4A7C15ull);
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)((z >> 11) + 1ull) * 0x1p-53;
}

/* transmission delay (an addition to the reference, whose synapses act in
 * the interval of the event): the event detected now enters bit 0 of the
 * synapse's ring, and the one detected delay intervals ago drives it */
static int net_delayed(orc_net *n, int k, int f_now) {
  unsigned long long r = (n->ring[k] << 1) | (unsigned long long)f_now;
  n->ring[k] = r;
  return (int)((r >> n->delay[k]) & 1ull);
}

int orc_net_set_delays(orc_net *n, int first, int count, const int *delay) {
  if (first < 0 || count < 0 || first + count > n->n) return -1;
  for (int i = 0; i < count; i++) {
    if (delay[i] < 0 || delay[i] > 63) return -1;
    n->delay[first + i] = delay[i];
  }
  return 0;
}

/* mfgr_update, grgo_update, gogr_update, grpkj_update (syn.cu:86-111,
 * 263-288, 412-437, 646-668); conductances syn.cuh:11-45 */
static void net_syn_update(orc_net *n, double t) {
  for (int k = 0; k < n->n; k++) {
    int kind = n->kind[k];
    if (kind == SYN_MFGR) {
      const double *r = n->rate[n->grp[k]];
      double fr = (r[2] <= t && t < r[3]) ? r[1] : r[0];
      double u = syn_uniform(n->seed[n->grp[k]], k, n->interval);
      int f = net_delayed(n, k, (fr * 0.125 * 0.001 > u) ? 1 : 0);
      double ampa = n->s0[k] * n->decay[0] + f;
      double nmda = ampa * n->decay[1] + f; /* from the updated AMPA, syn.cu:104 */
      n->s0[k] = ampa;
      n->s1[k] = nmda;
      n->val[k] = n->w[k] * (0.18e-9 * ampa + 0.025e-9 * nmda);
      continue;
    }
    double pv = n->sys[n->pre_sys[k]]->v[n->pre_comp[k]];
    int f = net_delayed(n, k, (pv > 0.0 && n->old_v[k] < 0.0) ? 1 : 0);
    if (kind == SYN_GRGO) {
      double a = n->s0[k] * n->decay[2] + f;
      double n1 = n->s1[k] * n->decay[3] + f;
      double n2 = n->s2[k] * n->decay[4] + f;
      n->s0[k] = a; n->s1[k] = n1; n->s2[k] = n2;
      n->val[k] = n->w[k] * (45.5e-9 * a + 30.0e-9 * (0.33 * n1 + 0.67 * n2));
    } else if (kind == SYN_GOGR) {
      double ga = n->s0[k] * n->decay[5] + f;
      double gb = n->s1[k] * n->decay[6] + f;
      n->s0[k] = ga; n->s1[k] = gb;
      n->val[k] = n->w[k] * 0.028e-9 * (0.43 * ga + 0.57 * gb);
    } else {
      double a = n->s0[k] * n->decay[7] + f;
      n->s0[k] = a;
      n->val[k] = a * n->w[k] * 0.7e-9;
    }
    n->old_v[k] = pv;
  }
  n->interval++;
}

/* one interval: every system in the order added, then the synapses */
int orc_net_advance(orc_net *n, double t) {
  for (int q = 0; q < n->nsys; q++) {
    int rc = orc_advance(n->sys[q], t);
    if (rc) return rc;
  }
  net_syn_update(n, t);
  return 0;
}

int orc_net_nsyn(const orc_net *n) { return n->n; }
const double *orc_net_syn(const orc_net *n, int field) {
  switch (field) {
    case 0: return n->val;
    case 1: return n->s0;
    case 2: return n->s1;
    case 3: return n->s2;
    default: return n->old_v;
  }
}

void orc_net_destroy(orc_net *n) {
  if (!n) return;
  free(n->kind); free(n->grp); free(n->pre_sys); free(n->pre_comp); free(n->post_sys); free(n->post_comp);
  free(n->w); free(n->s0); free(n->s1); free(n->s2); free(n->val); free(n->old_v); free(n->e);
  free(n->ring); free(n->delay);
  free(n);
}

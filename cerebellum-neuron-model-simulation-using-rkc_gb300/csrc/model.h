// Model constants of the four cerebellar cell types and the slot orders of
// their gating / conductance state, restated from the reference headers
// (param.h, gr.cuh, go.cuh, pkj.cuh, io.cuh, solve_rkc.cuh).  Shared by host
// and device code; plain C++ (no CUDA types) so the host setup can use it.
#pragma once

namespace gbrkc {

enum CellType { GR = 0, GO = 1, PKJ = 2, IO = 3, NTYPES = 4 };

constexpr double H_MAX = 0.125;        // one output interval, ms (param.h:12)
constexpr double UROUND = 2.22e-16;    // solve_rkc.cuh:22

// granule cell (gr.cuh:15-27)
constexpr double V_LEAK1_GR = -16.5, V_LEAK2_GR = -65.0, V_LEAK3_GR = -74.5;
constexpr double V_Na_GR = 87.39, V_K_GR = -84.69, V_Ca_GR = 129.33, V_INIT_GR = -80.0;
constexpr double Ca1_0_GR = 1e-4;
// Golgi cell (go.cuh:28-41)
constexpr double V_INIT_GO = -60.0, V_LEAK_GO = -55.0, V_Na_GO = 87.39, V_K_GO = -84.69;
constexpr double V_Ca_GO = 120.0, V_H_GO = -20.0, SHELL1_D_GO = 0.2e-4, B_Ca1_GO = 1.3;
constexpr double Ca1_0_GO = 5e-5, Ca1OUT_GO = 2.0, F_GO = 9.6485e4, G_GJ_GO = 2.5e-6;
// Purkinje cell (pkj.cuh:20-83)
constexpr double V_INIT_PKJ = -68.0, V_LEAK_PKJ = -80.0, V_Na_PKJ = 45.0, V_Ca_PKJ = 135.0;
constexpr double V_KH_PKJ = -30.0, V_K_PKJ = -85.0, G_GJ_PKJ = 2.5e-6;
constexpr double PKJ_SPINE_DENS = 13.0e4, PKJ_SPINE_AREA = 1.33e-8, PKJ_CM = 1.64;
constexpr double PKJ_RM_S = 10.0, PKJ_RM_D = 30.0, PKJ_RI = 0.25, B_Ca1_PKJ = 10.0;
constexpr double PKJ_SHELLD = 0.2e-4, Ca1OUT_PKJ = 2.4, Ca1_0_PKJ = 4.0e-5, F_PKJ = 9.6485e4;
// inferior olive (io.cuh:16-51)
constexpr double V_INIT_IO = -60.0, V_LEAK_IO = 10.0, V_Na_IO = 55.0, V_Ca_IO = 120.0;
constexpr double V_K_IO = -75.0, V_H_IO = -43.0, G_INT_IO = 0.13, G_P_DS_IO = 0.200;
constexpr double G_P_SA_IO = 0.869, G_C_IO = 0.04, CA_PH_IO = 3.0, BETA_CA_IO = 0.075;

// per-type RKC tolerance and minimum step (solve_rkc.cuh:24-31)
constexpr double TOL_DEFAULT[4] = {1.0e-9, 1.0e-6, 1.0e-6, 1.0e-6};
constexpr int HMIN_LOG2_DEFAULT[4] = {-12, -10, -10, -10};

// gating-state slots (gr.cuh:35-37, go.cuh:47-51, pkj.cuh:86-88, io.cuh:56-57)
enum GrIon { GR_n_KV, GR_a_KA, GR_b_KA, GR_c_KCa, GR_s_KM, GR_ir_KIR, GR_ch_Ca, GR_ci_Ca,
             GR_o_Na, GR_c1, GR_c2, GR_c3, GR_c4, GR_c5, GR_i1, GR_i2, GR_i3, GR_i4, GR_i5,
             GR_i6, GR_NION };
enum GoIon { GO_m_NaT, GO_h_NaT, GO_r_NaR, GO_s_NaR, GO_p_NaP, GO_n_KV, GO_a_KA, GO_b_KA,
             GO_c_KC, GO_sl, GO_ch, GO_ci, GO_cl, GO_cm, GO_hf1, GO_hf2, GO_hs1, GO_hs2,
             GO_o1, GO_o2, GO_c1, GO_c2, GO_c3, GO_c4, GO_NION };
enum PkIon { PK_m_NaF, PK_h_NaF, PK_m_NaP, PK_m_CaP, PK_h_CaP, PK_m_CaT, PK_h_CaT, PK_m_KA,
             PK_h_KA, PK_m_KC, PK_m_Kh1, PK_m_Kh2, PK_m_Kdr, PK_h_Kdr, PK_m_KM, PK_z_KC,
             PK_m_K2, PK_z_K2, PK_NION };
enum IoIon { IO_k, IO_l, IO_m, IO_h, IO_n, IO_p, IO_x, IO_r, IO_s, IO_q, IO_NION };
// conductance slots (gr.cuh:39-40, go.cuh:53-54, pkj.cuh:91-92, io.cuh:59)
enum GrCond { GR_g_leak1, GR_g_leak2, GR_g_leak3, GR_g_Na, GR_g_KV, GR_g_KA, GR_g_KCa,
              GR_g_KM, GR_g_KIR, GR_g_Ca, GR_NCOND };
enum GoCond { GO_g_leak, GO_g_NaT, GO_g_NaR, GO_g_NaP, GO_g_KV, GO_g_KA, GO_g_KC, GO_g_Kslow,
              GO_g_CaHVA, GO_g_CaLVA, GO_g_HCN1, GO_g_HCN2, GO_g_KAHP, GO_NCOND };
enum PkCond { PK_g_leak, PK_g_NaF, PK_g_NaP, PK_g_CaP, PK_g_CaT, PK_g_Kh, PK_g_Kdr, PK_g_KM,
              PK_g_KA, PK_g_KC, PK_g_K2, PK_NCOND };
enum IoCond { IO_g_leak, IO_g_CaL, IO_g_Na, IO_g_Kdr, IO_g_K, IO_g_CaH, IO_g_KCa, IO_g_H,
              IO_NCOND };

constexpr int NION[4] = {GR_NION, GO_NION, PK_NION, IO_NION};
constexpr int NCOND[4] = {GR_NCOND, GO_NCOND, PK_NCOND, IO_NCOND};
constexpr int ROW_FIELDS[4] = {17, 20, 7, 6};

// Granule Na Markov parameters per compartment type (gr_ion.cu:56-70); the
// host fills a, b = (Oon/Con)^(1/4), (Ooff/Coff)^(1/4) and their 4th powers.
struct NaPar {
  double n1, n2, n3, n4, Aa, Ab, vshift, Con, Coff, Oon, Ooff, a, b, a4, b4;
};

}  // namespace gbrkc

// Host runtime of the RKC engine: model setup from reference-format
// morphology rows (the reference's initialize_host_* and set_host_*_solve:
// gr.cu:3-82, go.cu:3-88, pkj.cu:3-169, io.cu:3-102, *_solve.cu), packing of
// systems into per-type pools, the Chebyshev coefficient table, device
// allocation, and the C ABI of include/gbrkc.h.
//
// Built with -ffp-contract=off: the static per-compartment values (areas,
// capacitances, conductances, axial conductances) are computed in the same
// operation order as the reference, so they are bit-identical on every host.
#include <cuda_runtime.h>
#include <limits.h>
#include <math.h>
#include <stdarg.h>
#include <stdlib.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <type_traits>
#include <memory>
#include <string>
#include <vector>

#include "../../include/gbrkc.h"
#include "engine.h"
#include "host_init.h"
#include "model.h"
#include "noalloc.h"

namespace gbrkc {

static thread_local std::string g_last_error;

// GBRKC_MIXED_GR=fp64 keeps FP64 gating for granule pools in a mixed
// engine.  A granule cell's step decisions (tolerance 1e-9) follow the last
// bits of its channel currents, and a different decision moves its voltage
// by up to ~0.1 mV within a millisecond; with FP64 gating its results are
// the FP64 engine's, bit for bit, at the cost of its FP64 Markov and gating
// updates (about half the mixed batch's throughput).
bool mixed_granules_fp64() {
  const char *v = getenv("GBRKC_MIXED_GR");
  return v && (strcmp(v, "fp64") == 0 || strcmp(v, "FP64") == 0);
}

static int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

// A C entry point lets no C++ exception out: host allocations sized by the
// caller (dense templates, recorders, logs) report GBRKC_ENOMEM instead.
template <class F>
static int no_throw(F &&f) {
  try {
    return f();
  } catch (const std::bad_alloc &) {
    return fail(GBRKC_ENOMEM, "host memory exhausted");
  } catch (const std::exception &x) {
    return fail(GBRKC_EINVAL, "%s", x.what());
  }
}

#define CUDA_TRY(x)                                                                     \
  do {                                                                                  \
    cudaError_t e_ = (x);                                                               \
    if (e_ != cudaSuccess) return fail(GBRKC_ECUDA, "%s: %s", #x, cudaGetErrorString(e_)); \
  } while (0)

// ------------------------------------------------------------------ setup
struct Template {
  int type, ncomp;
  std::vector<double> rows;
  std::vector<double> area, cm, shell, invcm;
  std::vector<int> ctype;
  std::vector<std::vector<double>> cond;  // [k][comp]
  // CSR of one cell with the diagonal kept (RKC sign), as the reference builds it
  std::vector<int> row, col;
  std::vector<double> val;
};

struct HostSystem {
  int type, nx, ny, n, ncomp, nc;
  int tmpl;
  bool gap;
  std::vector<int> gj_pairs;
  std::vector<double> io_gap_g, jitter;
  std::vector<int> stim_comp;
  std::vector<double> stim_amp, stim_t0, stim_t1;
  std::vector<double> cond_scale;             // per cell, empty: 1
  std::vector<double> cond_scale_ch;          // per cell and channel (replaces cond_scale), empty: none
  double tol, hmin;
  bool idle = false;                          // a free slot until reset
  // built
  int csr = -1;                               // index into the system-CSR table
  std::vector<int> gap_pre, gap_post;
  std::vector<double> gap_g;
  int pool_index = -1;
};

static double row_f(const std::vector<double> &r, int nf, int i, int f) { return r[(size_t)i * nf + f]; }

// one cell of a type from its rows (initialize_host_* + the dense axial matrix)
static int make_template(int type, int ncomp, const double *rows, Template &T) {
  const int nf = ROW_FIELDS[type];
  T.type = type;
  T.ncomp = ncomp;
  T.rows.assign(rows, rows + (size_t)ncomp * nf);
  T.area.assign(ncomp, 0.0);
  T.cm.assign(ncomp, 0.0);
  T.shell.assign(ncomp, 0.0);
  T.ctype.assign(ncomp, 0);
  T.cond.assign(NCOND[type], std::vector<double>(ncomp, 0.0));
  std::vector<double> rad(ncomp), len(ncomp), Ra(ncomp), mat((size_t)ncomp * ncomp, 0.0);
  std::vector<int> parent(ncomp);
  // Purkinje channel densities per class (pkj.cuh:29-65): NaF NaP CaP CaT KH KDR KM KA KC K2
  static const double Gpk[4][10] = {{7500.0, 1.0, 0.0, 0.5, 0.3, 600.0, 0.040, 15.0, 0.0, 0.0},
                                    {0.0, 0.0, 4.5, 0.5, 0.0, 60.0, 0.01, 2.0, 80.0, 0.39},
                                    {0.0, 0.0, 4.5, 0.5, 0.0, 0.0, 0.013, 0.0, 80.0, 0.39},
                                    {0.0, 0.0, 4.5, 0.5, 0.0, 0.0, 0.013, 0.0, 80.0, 0.39}};
  // inferior-olive densities per class (io.cu:48-82)
  static const double Gio[3][8] = {{0.016 / (1 * 1.0), 0.0, 0.0, 0.0, 0.0, 4.5 / (1 * 1.0), 35.0 / (1 * 1.0), 0.15 / (1 * 1.0)},
                                   {0.016, 0.83, 120.0, 9.0, 5.0, 0.0, 0.0, 0.0},
                                   {0.016, 0.0, 240.0, 0.0, 20.0, 0.0, 0.0, 0.0}};
  for (int i = 0; i < ncomp; i++) {
    if ((int)row_f(T.rows, nf, i, 0) != i) return fail(GBRKC_EINVAL, "morphology row %d has index %d", i, (int)row_f(T.rows, nf, i, 0));
    parent[i] = (int)row_f(T.rows, nf, i, 1);
    if (parent[i] < -1 || parent[i] >= ncomp || parent[i] == i)
      return fail(GBRKC_EINVAL, "morphology row %d has parent %d", i, parent[i]);
    if (type == GR || type == GO) {
      double d1 = row_f(T.rows, nf, i, 2), d2 = row_f(T.rows, nf, i, 3), d3 = row_f(T.rows, nf, i, 4), d4 = row_f(T.rows, nf, i, 5);
      int i3 = (int)row_f(T.rows, nf, i, 6);
      if (i3 < 0 || i3 > 8) return fail(GBRKC_EINVAL, "compartment type %d out of range", i3);
      rad[i] = 0.5 * d1 * 1e-4; len[i] = d2 * 1e-4; Ra[i] = d3 * 1e-3;
      T.ctype[i] = i3;
      T.area[i] = 2.0 * M_PI * rad[i] * len[i];
      double a = T.area[i];
      T.cm[i] = d4 * a;
      for (int k = 0; k < NCOND[type]; k++) T.cond[k][i] = row_f(T.rows, nf, i, 7 + k) * a;
    } else if (type == PKJ) {
      double x = row_f(T.rows, nf, i, 2), y = row_f(T.rows, nf, i, 3), z = row_f(T.rows, nf, i, 4), dd = row_f(T.rows, nf, i, 5);
      int i3 = (int)row_f(T.rows, nf, i, 6);
      if (i3 < 0 || i3 > 3) return fail(GBRKC_EINVAL, "Purkinje compartment type %d out of range", i3);
      double a;
      rad[i] = 0.5 * dd * 1e-4;
      Ra[i] = PKJ_RI;
      T.ctype[i] = i3;
      if (i3 == 0) {
        len[i] = dd * 1e-4;
        T.area[i] = 4.0 * M_PI * rad[i] * rad[i];
        a = T.area[i];
        T.cm[i] = PKJ_CM * a;
        T.shell[i] = (PKJ_SHELLD - 2 * pow(PKJ_SHELLD, 2) / (dd * 1e-4) + 4 * pow(PKJ_SHELLD, 3) / (3 * pow(dd * 1e-4, 2))) * T.area[i];
        T.cond[PK_g_leak][i] = 1.0 / PKJ_RM_S * a;
      } else {
        len[i] = sqrt(pow(x, 2) + pow(y, 2) + pow(z, 2)) * 1e-4;
        T.area[i] = 2.0 * M_PI * rad[i] * len[i];
        a = T.area[i];
        T.shell[i] = (PKJ_SHELLD - pow(PKJ_SHELLD, 2) / (dd * 1e-4)) * T.area[i];
        if (i3 == 3) {
          double other = a + len[i] * PKJ_SPINE_AREA * PKJ_SPINE_DENS;
          T.cm[i] = PKJ_CM * other;
          T.cond[PK_g_leak][i] = 1.0 / PKJ_RM_D * other;
        } else {
          T.cm[i] = PKJ_CM * a;
          T.cond[PK_g_leak][i] = 1.0 / PKJ_RM_D * a;
        }
      }
      for (int k = 0; k < 10; k++) T.cond[1 + k][i] = Gpk[i3][k] * a;
    } else {
      double d1 = row_f(T.rows, nf, i, 2), d2 = row_f(T.rows, nf, i, 3), d4 = row_f(T.rows, nf, i, 4);
      int i3 = (int)row_f(T.rows, nf, i, 5);
      if (i3 < 0 || i3 > 2) return fail(GBRKC_EINVAL, "IO compartment type %d out of range", i3);
      rad[i] = 0.5 * d1 * 1e-4; len[i] = d2 * 1e-4;
      T.ctype[i] = i3;
      T.area[i] = 2.0 * M_PI * rad[i] * len[i];
      T.cm[i] = d4;
      for (int k = 0; k < 8; k++) T.cond[k][i] = Gio[i3][k];
    }
  }
  if (type == IO) {
    // io_solve.cu:37-65: asymmetric dendrite / soma / axon coupling
    for (int i = 0; i < ncomp; i++) {
      int d = parent[i], i3 = T.ctype[i];
      double lg = 0.0, lgr = 0.0;
      if (d >= 0) {
        if (i3 == 0 && d == 1) { lg = (G_INT_IO / (1.0 - G_P_DS_IO)); lgr = (G_INT_IO / (G_P_DS_IO)); }
        else if (i3 == 1 && d == 2) { lg = (G_INT_IO / (G_P_SA_IO)); lgr = (G_INT_IO / (1.0 - G_P_SA_IO)); }
        else if (i3 == 0 && d < 1) { lg = lgr = (G_INT_IO / (0.5)); }
        mat[d + (size_t)ncomp * i] = lg;
        mat[i + (size_t)ncomp * d] = lgr;
      }
    }
  } else {
    // gr_solve.cu:37-43 and siblings: 2 / (R_i + R_parent) with R = Ra len / (pi r^2)
    for (int i = 0; i < ncomp; i++) {
      int d = parent[i];
      if (d >= 0) {
        mat[d + (size_t)ncomp * i] = (2.0 / ((Ra[i] * len[i]) / (rad[i] * rad[i] * M_PI) + (Ra[d] * len[d]) / (rad[d] * rad[d] * M_PI)));
        mat[i + (size_t)ncomp * d] = mat[d + (size_t)ncomp * i];
      }
    }
  }
  // dense -> CSR with explicit diagonal, values in the RKC sign convention
  // (pkj_solve.cu:152-183 then 244-251): off-diagonal +g, diagonal -(sum g)
  T.row.assign(ncomp + 1, 0);
  T.col.clear();
  T.val.clear();
  for (int r = 0; r < ncomp; r++) {
    int dig = -1;
    for (int c = 0; c < ncomp; c++) {
      double m = mat[(size_t)r * ncomp + c];
      if (m > 0.0) { T.val.push_back(-m); T.col.push_back(c); }
      else if (r == c) { dig = (int)T.val.size(); T.val.push_back(0.0); T.col.push_back(c); }
    }
    for (int c = 0; c < ncomp; c++)
      if (c != r) T.val[dig] += mat[(size_t)r * ncomp + c];
    T.row[r + 1] = (int)T.val.size();
  }
  for (double &v : T.val) v = -v;
  T.invcm.resize(ncomp);
  for (int i = 0; i < ncomp; i++) T.invcm[i] = 1.0 / T.cm[i];
  return 0;
}

// full system CSR of a multi-cell GO/PKJ system with its linear gap junctions
// (go_solve.cu:51-81,160-196; pkj_solve.cu:4-26,79-120,200-236)
struct SysCsr {
  std::vector<int> row, col;
  std::vector<double> val, invcm;
};

static int build_system_csr(const HostSystem &S, const Template &T, SysCsr &C) {
  const int N = S.ncomp, n = S.n, nc = S.nc;
  std::vector<int> gpre, gpost;
  double ggj = 0.0;
  if (S.type == GO) {
    int gx = S.nx, gy = S.ny;
    for (int y = 0; y < gy; y++)
      for (int x = 0; x < gx - 1; x++) { gpre.push_back((y * gx + x) * N); gpre.push_back((y * gx + x + 1) * N); }
    for (int x = 0; x < gx; x++)
      for (int y = 0; y < gy - 1; y++) { gpre.push_back((y * gx + x) * N); gpre.push_back(((y + 1) * gx + x) * N); }
    ggj = G_GJ_GO;
  } else {
    int px = S.nx, py = S.ny, G = (int)S.gj_pairs.size() / 2;
    for (int y = 0; y < py; y++)
      for (int x = 0; x < px - 1; x++)
        for (int i = 0; i < G; i++) {
          int a = S.gj_pairs[2 * i], b = S.gj_pairs[2 * i + 1];
          if (a < 0 || a >= N || b < 0 || b >= N) return fail(GBRKC_EINVAL, "gap-junction pair (%d,%d) out of range", a, b);
          gpre.push_back(a + (x + y * px) * N);
          gpre.push_back(b + ((x + 1) + y * px) * N);
        }
    ggj = G_GJ_PKJ;
  }
  const int n_gj = (int)gpre.size();
  gpost.assign(n_gj, 0);
  for (int i = 0; i < n_gj; i += 2) { gpost[i + 1] = gpre[i]; gpost[i] = gpre[i + 1]; }
  const int nnz_cell = (int)T.val.size();
  C.row.assign(nc + 1, 0);
  C.col.assign((size_t)nnz_cell * n + n_gj, 0);
  C.val.assign((size_t)nnz_cell * n + n_gj, 0.0);
  for (int ci = 0; ci < n; ci++) {
    for (int j = 0; j < nnz_cell; j++) {
      C.val[j + (size_t)nnz_cell * ci] = T.val[j];
      C.col[j + (size_t)nnz_cell * ci] = T.col[j] + N * ci;
    }
    for (int j = 0; j < N; j++) C.row[j + N * ci] = T.row[j] + nnz_cell * ci;
  }
  C.row[nc] = nnz_cell * n;
  for (int i = 0; i < n_gj; i++) {
    const int pre = gpre[i], post = gpost[i];
    for (int j = C.row[pre]; j < C.row[pre + 1]; j++)
      if (C.col[j] == pre) { C.val[j] -= ggj; break; }
    int pos = C.row[pre + 1];
    for (int j = C.row[pre]; j < C.row[pre + 1]; j++) {
      if (C.col[j] == post) return fail(GBRKC_EINVAL, "duplicate gap junction %d->%d", pre, post);
      if (C.col[j] > post) { pos = j; break; }
    }
    const int used = C.row[nc];
    for (int j = used; j > pos; j--) { C.col[j] = C.col[j - 1]; C.val[j] = C.val[j - 1]; }
    C.col[pos] = post;
    C.val[pos] = ggj;
    for (int r = pre + 1; r <= nc; r++) C.row[r]++;
  }
  C.invcm.resize(nc);
  for (int i = 0; i < nc; i++) C.invcm[i] = T.invcm[i % N];
  return 0;
}

// IO nonlinear gap network (gap.cu:4-120), including idy = id / ny
static int build_io_gap(HostSystem &S) {
  const int nx = S.nx, ny = S.ny, n = S.n;
  if (nx != ny) return fail(GBRKC_EINVAL, "IO gap network needs a square grid (the reference indexes rows by id / ny)");
  S.gap_pre.assign(4 * n, 0);
  S.gap_post.assign(4 * n, 0);
  S.gap_g.assign(4 * n, G_C_IO);
  for (int id = 0; id < n; id++) {
    int idx = id % nx, idy = id / ny;
    int L = id - 1, U = id - nx, R = id + 1, D = id + nx;
    if (idx == 0 && idy == 0) { L = -1; U = -1; }
    else if (idx == nx - 1 && idy == 0) { U = -1; R = -1; }
    else if (idx == 0 && idy == ny - 1) { L = -1; D = -1; }
    else if (idx == nx - 1 && idy == ny - 1) { R = -1; D = -1; }
    else if (idy == 0) { U = -1; }
    else if (idy == ny - 1) { D = -1; }
    else if (idx == 0) { L = -1; }
    else if (idx == nx - 1) { R = -1; }
    const int nb[4] = {L, U, R, D};
    for (int k = 0; k < 4; k++) {
      if (nb[k] >= n) return fail(GBRKC_EINVAL, "IO gap neighbour out of range");
      S.gap_post[id * 4 + k] = id * S.ncomp;
      S.gap_pre[id * 4 + k] = nb[k] * S.ncomp;
      if (!S.io_gap_g.empty()) S.gap_g[id * 4 + k] = S.io_gap_g[id * 4 + k];
    }
  }
  return 0;
}

// Chebyshev stage coefficients per stage count m, computed exactly as the
// reference's step() does (solve_rkc.cu:826-870), so the device reproduces
// them bit for bit without transcendental functions.
static void coef_table(int mmax, std::vector<double> &coef, std::vector<long> &off) {
  off.assign(mmax + 2, 0);
  coef.clear();
  for (int m = 1; m <= mmax; m++) {
    off[m] = (long)coef.size();
    double w0 = 1.0 + 2.0 / (13.0 * m * m);
    double temp1 = w0 * w0 - 1.0;
    double temp2 = sqrt(temp1);
    double arg = m * log(w0 + temp2);
    double w1 = sinh(arg) * temp1 / (cosh(arg) * m * temp2 - w0 * sinh(arg));
    double bjm1 = 1.0 / ((2.0 * w0) * (2.0 * w0));
    double bjm2 = bjm1;
    double mus = w1 * bjm1;
    coef.push_back(mus);
    double zjm1 = w0, zjm2 = 1.0, dzjm1 = 1.0, dzjm2 = 0.0, d2zjm1 = 0.0, d2zjm2 = 0.0;
    for (int j = 1; j < m; j++) {
      double zj = 2.0 * w0 * zjm1 - zjm2;
      double dzj = 2.0 * w0 * dzjm1 - dzjm2 + 2.0 * zjm1;
      double d2zj = 2.0 * w0 * d2zjm1 - d2zjm2 + 4.0 * dzjm1;
      double bj = d2zj / (dzj * dzj);
      double ajm1 = 1.0 - zjm1 * bjm1;
      double mu = 2.0 * w0 * bj / bjm1;
      double nu = -bj / bjm2;
      mus = mu * w1 / w0;
      coef.push_back(mu);
      coef.push_back(nu);
      coef.push_back((1.0 - mu - nu));
      coef.push_back(mus);
      coef.push_back(ajm1);
      bjm2 = bjm1; bjm1 = bj; zjm2 = zjm1; zjm1 = zj; dzjm2 = dzjm1; dzjm1 = dzj;
      d2zjm2 = d2zjm1; d2zjm1 = d2zj;
    }
  }
  off[mmax + 1] = (long)coef.size();
}

// ----------------------------------------------------------------- pools
struct DeviceMem {
  std::vector<void *> ptrs;
  std::vector<size_t> sizes;   // bytes of each allocation (gbrkc_autotune's snapshots)
  ~DeviceMem() {
    for (void *p : ptrs) cudaFree(p);
  }
  template <typename T>
  int upload(const std::vector<T> &h, T **d) {
    size_t bytes = std::max<size_t>(h.size(), 1) * sizeof(T);
    cudaError_t e = cudaMalloc((void **)d, bytes);
    if (e != cudaSuccess) return fail(GBRKC_ENOMEM, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
    ptrs.push_back(*d);
    sizes.push_back(bytes);
    if (!h.empty()) {
      e = cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
      if (e != cudaSuccess) return fail(GBRKC_ECUDA, "cudaMemcpy: %s", cudaGetErrorString(e));
    }
    return 0;
  }
};

struct PoolHost {
  int type;
  bool f64 = false;                    // the pool's gating arithmetic: FP64 (vd) or FP32 (vf)
  std::vector<int> systems;            // engine system ids
  long nc = 0;
  int ncell = 0;
  // per system
  std::vector<int> sys_off, sys_nc, sys_ncell, sys_ncomp, sys_tmpl, sys_csr, sys_cell0, sys_gap0, sys_ngap;
  std::vector<long> sys_ws;
  std::vector<Ctl> ctl;
  // per compartment
  std::vector<double> v, ca, ca2, rev, ca_old, iext, shell, area, ion, cond;
  std::vector<uint8_t> ctype, flags;
  // templates used by this pool
  std::vector<int> t_row0, t_nz0, t_cm0, t_row, t_col;
  std::vector<double> t_g, t_invcm, t_gc, t_Gc;
  std::map<int, int> tmpl_local;
  std::vector<int> s_row0, s_nz0, s_cm0, s_row, s_col;
  std::vector<double> s_g, s_invcm, s_gc, s_Gc;
  std::vector<int> gap_pre, gap_post;
  std::vector<double> gap_g;
  std::vector<int> stim_comp, cell_soma, cell_spk;
  std::vector<int> cell_sys, cell_local;  // per pool cell: engine system id, cell within it
  std::vector<double> stim_amp, stim_t0, stim_t1;
  long ws_total = 0;
  int max_nc = 0, min_nc = 1 << 30, max_ncell = 0;
  // launch configuration
  int team = TEAM_BLOCK, block = 256, grid = 1;
  int grid_bw = GRID_BLOCK;                 // grid team: threads of each CTA that own elements
  int grid_rl = 0, grid_maxdeg = 0;         // grid team: row slots per CTA, entries per slot (0: no copy)
  std::vector<int> grid_nbr;                // grid team: neighbour CTAs per CTA (empty: grid barriers only)
  unsigned long long *d_grid_flags = nullptr;
  size_t smem = 0;
  int ws_in_smem = 0;
  long ws_tile = 0;
  // device views
  PoolView<double> vd{};
  PoolView<float> vf{};
  double *d_ws = nullptr, *d_vnew = nullptr, *d_v = nullptr, *d_ca = nullptr, *d_rev = nullptr, *d_ede = nullptr;
  void *d_ion = nullptr;
  Ctl *d_ctl = nullptr;
  double *d_soma = nullptr;
  int soma_cap = 0;
  int rec_w = 1;                         // compartments recorded per cell
  int *d_cell_soma = nullptr;
  double *d_spk_prev = nullptr;
  SpikeRec *d_spk_log = nullptr;         // owned here (re-sized by gbrkc_record_spikes)
  int *d_spk_count = nullptr;
  unsigned *d_grid_bar = nullptr;        // grid team: the barrier's words (zeroed before each launch)
  int spk_cap = 0;
  std::vector<char> retired;
};

}  // namespace gbrkc

using namespace gbrkc;

struct gbrkc_engine {
  int precision = GBRKC_FP64;
  bool gr_f64 = false;                 // mixed precision: granule pools keep FP64 gating (GBRKC_MIXED_GR=fp64)
  bool built = false;
  std::vector<Template> templates;
  std::map<std::pair<int, std::vector<double>>, int> tmpl_index;
  std::vector<HostSystem> systems;
  std::vector<SysCsr> csrs;
  PoolHost pools[NTYPES];
  DeviceMem mem;
  cudaStream_t streams[NTYPES] = {};
  std::vector<double> coef;
  std::vector<long> coef_off;
  double *d_coef = nullptr;
  long *d_coef_off = nullptr;
  int coef_mmax = 0;
  int soma_cap = 0;
  int soma_iv = 0;   // intervals recorded so far
  int n_retired = 0;
  bool pending_init = false;    // systems reset since the last launch wait for initialisation
  cudaEvent_t ev_start = nullptr, ev_end = nullptr, ev_k0[NTYPES] = {}, ev_k1[NTYPES] = {};
  float last_ms = 0.0f, last_kernel_ms[NTYPES] = {};
  // persistent mixed-type launch
  bool mega = false;
  int mega_grid = 0;
  size_t mega_smem = 0;
  int role_ctas[NTYPES] = {};
  int role_cap[NTYPES] = {};
  int gr_warps = 0;             // granule warps of the next launch (32 lanes each)
  int gr_warps_need = 0;        // granule warps that would give every granule system with work its own lane
  int gr_warps_max = 0;         // granule warps the CTAs can hold beside the other roles
  int lanes = 16;               // lanes of a warp that take single-lane systems
  long gr_active = -1;          // granule systems with work (-1: not known yet)
  double role_work[NTYPES] = {};  // smoothed CTA-ms per role
  int *d_queue = nullptr;
  unsigned long long *d_tstart = nullptr, *d_tend = nullptr;
  // device address of noalloc.cu's static launch scratch, looked up at build
  // on the engine's device (persistent engines only)
  unsigned long long *d_static_scratch = nullptr;
  // chemical synapses (network mode), as added
  struct {
    std::vector<int> kind, grp, pre_sys, pre_comp, post_sys, post_comp;
    std::vector<unsigned char> delay;
    std::vector<double> w, grp_rate;
    std::vector<unsigned long long> grp_seed;
  } syn;
  SynView sv{};
  long long syn_interval = 0;   // intervals advanced in network mode (Poisson counter)
  ~gbrkc_engine() {
    for (auto &P : pools)
      if (P.d_spk_log) cudaFree(P.d_spk_log);
    for (auto &s : streams)
      if (s) cudaStreamDestroy(s);
    for (cudaEvent_t e : {ev_start, ev_end})
      if (e) cudaEventDestroy(e);
    for (int t = 0; t < NTYPES; t++) {
      if (ev_k0[t]) cudaEventDestroy(ev_k0[t]);
      if (ev_k1[t]) cudaEventDestroy(ev_k1[t]);
    }
  }
};

extern "C" const char *gbrkc_last_error(void) { return g_last_error.c_str(); }

extern "C" int gbrkc_engine_create(int precision, gbrkc_engine **out) {
  if (!out || (precision != GBRKC_FP64 && precision != GBRKC_MIXED)) return fail(GBRKC_EINVAL, "bad arguments");
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) return fail(GBRKC_ECUDA, "no CUDA device: %s", cudaGetErrorString(e));
  std::unique_ptr<gbrkc_engine> E(new gbrkc_engine());
  E->precision = precision;
  E->gr_f64 = precision == GBRKC_MIXED && mixed_granules_fp64();
  // lanes per warp that take single-lane systems: fewer systems in a warp
  // diverge less but need more warps (measured on the GB300: 1024 granule
  // cells on 32 SMs took 115 / 103 / 95 ms per simulated ms with 32 / 16 / 8
  // lanes; the mixed workload's persistent launch 596 / 574 / 628 / 1135 ms
  // per 5 ms with 32 / 16 / 8 / 4 in mixed precision, while in FP64 16 lanes
  // were slower than 32); GBRKC_LANES overrides
  E->lanes = (precision == GBRKC_MIXED) ? 16 : 32;
  if (const char *l = getenv("GBRKC_LANES")) E->lanes = std::max(1, std::min(32, atoi(l)));
  for (auto &s : E->streams) CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  CUDA_TRY(cudaEventCreate(&E->ev_start));
  CUDA_TRY(cudaEventCreate(&E->ev_end));
  for (int t = 0; t < NTYPES; t++) {
    CUDA_TRY(cudaEventCreate(&E->ev_k0[t]));
    CUDA_TRY(cudaEventCreate(&E->ev_k1[t]));
  }
  *out = E.release();
  return 0;
}

extern "C" void gbrkc_engine_destroy(gbrkc_engine *e) { delete e; }

static int add_system_impl(gbrkc_engine *E, const gbrkc_system_desc *d, int *sys_id) {
  if (!E || !d || !d->rows || !d->jitter) return fail(GBRKC_EINVAL, "null argument");
  if (E->built) return fail(GBRKC_ESTATE, "engine already built");
  if (d->cell_type < 0 || d->cell_type >= NTYPES || d->nx <= 0 || d->ny <= 0 || d->ncomp <= 0)
    return fail(GBRKC_EINVAL, "bad system shape");
  // compartment indices are 32-bit on the device
  if ((long long)d->nx * d->ny * d->ncomp > (long long)INT_MAX / 2)
    return fail(GBRKC_EINVAL, "system too large (%lld compartments)", (long long)d->nx * d->ny * d->ncomp);
  HostSystem S;
  S.type = d->cell_type; S.nx = d->nx; S.ny = d->ny; S.n = d->nx * d->ny; S.ncomp = d->ncomp;
  S.nc = S.n * S.ncomp;
  S.gap = d->gap_junctions != 0;
  const int nf = ROW_FIELDS[S.type];
  std::vector<double> rows(d->rows, d->rows + (size_t)d->ncomp * nf);
  auto key = std::make_pair(S.type, rows);
  auto it = E->tmpl_index.find(key);
  if (it == E->tmpl_index.end()) {
    Template T;
    int rc = make_template(S.type, S.ncomp, d->rows, T);
    if (rc) return rc;
    E->templates.push_back(std::move(T));
    it = E->tmpl_index.emplace(key, (int)E->templates.size() - 1).first;
  }
  S.tmpl = it->second;
  if (d->gj_pairs && d->n_gj_pairs > 0) S.gj_pairs.assign(d->gj_pairs, d->gj_pairs + 2 * d->n_gj_pairs);
  if (d->io_gap_g) S.io_gap_g.assign(d->io_gap_g, d->io_gap_g + 4 * (size_t)S.n);
  S.jitter.assign(d->jitter, d->jitter + S.n);
  S.stim_comp.assign(S.n, -1);
  S.stim_amp.assign(S.n, 0.0); S.stim_t0.assign(S.n, 0.0); S.stim_t1.assign(S.n, 0.0);
  if (d->stim_comp) {
    if (!d->stim_amp || !d->stim_t0 || !d->stim_t1) return fail(GBRKC_EINVAL, "incomplete stimulus");
    for (int c = 0; c < S.n; c++) {
      if (d->stim_comp[c] >= S.ncomp) return fail(GBRKC_EINVAL, "stimulus compartment out of range");
      S.stim_comp[c] = d->stim_comp[c];
      S.stim_amp[c] = d->stim_amp[c]; S.stim_t0[c] = d->stim_t0[c]; S.stim_t1[c] = d->stim_t1[c];
    }
  }
  if (d->cond_scale) {
    S.cond_scale.assign(d->cond_scale, d->cond_scale + S.n);
    for (double x : S.cond_scale)
      if (!(x >= 0.0) || !std::isfinite(x)) return fail(GBRKC_EINVAL, "conductance scale must be finite and >= 0");
  }
  if (d->cond_scale_ch) {
    S.cond_scale_ch.assign(d->cond_scale_ch, d->cond_scale_ch + (size_t)S.n * NCOND[S.type]);
    for (double x : S.cond_scale_ch)
      if (!(x >= 0.0) || !std::isfinite(x)) return fail(GBRKC_EINVAL, "conductance scale must be finite and >= 0");
  }
  S.idle = d->idle != 0;
  S.tol = d->tol > 0 ? d->tol : TOL_DEFAULT[S.type];
  S.hmin = d->hmin > 0 ? d->hmin : pow(2.0, (double)HMIN_LOG2_DEFAULT[S.type]);
  if (S.n > 1 && S.gap) {
    if (S.type == IO) {
      int rc = build_io_gap(S);
      if (rc) return rc;
    } else if (S.type == GO || (S.type == PKJ && !S.gj_pairs.empty())) {
      SysCsr C;
      int rc = build_system_csr(S, E->templates[S.tmpl], C);
      if (rc) return rc;
      E->csrs.push_back(std::move(C));
      S.csr = (int)E->csrs.size() - 1;
    }
  }
  if (S.n > 1 && S.csr < 0) {
    // multi-cell system without linear junctions: replicate the template into
    // a system CSR so the stage loop needs no cell arithmetic
    const Template &T = E->templates[S.tmpl];
    SysCsr C;
    const int nz = (int)T.val.size();
    C.row.assign(S.nc + 1, 0);
    C.col.resize((size_t)nz * S.n);
    C.val.resize((size_t)nz * S.n);
    for (int ci = 0; ci < S.n; ci++) {
      for (int j = 0; j < nz; j++) {
        C.col[j + (size_t)nz * ci] = T.col[j] + S.ncomp * ci;
        C.val[j + (size_t)nz * ci] = T.val[j];
      }
      for (int j = 0; j < S.ncomp; j++) C.row[j + S.ncomp * ci] = T.row[j] + nz * ci;
    }
    C.row[S.nc] = nz * S.n;
    C.invcm.resize(S.nc);
    for (int i = 0; i < S.nc; i++) C.invcm[i] = T.invcm[i % S.ncomp];
    E->csrs.push_back(std::move(C));
    S.csr = (int)E->csrs.size() - 1;
  }
  E->systems.push_back(std::move(S));
  if (sys_id) *sys_id = (int)E->systems.size() - 1;
  return 0;
}

extern "C" int gbrkc_add_system(gbrkc_engine *E, const gbrkc_system_desc *d, int *sys_id) {
  return no_throw([&] { return add_system_impl(E, d, sys_id); });
}

namespace {

// Systems of at least this many compartments run on a thread-block cluster
// (GBRKC_CLUSTER_MIN_NC overrides, e.g. to exercise the path on small cases).
int cluster_min_nc() {
  const char *v = getenv("GBRKC_CLUSTER_MIN_NC");
  if (v && v[0]) return atoi(v);
  return 4096;
}

// Whether pool P is one system of at least cluster_min_nc() compartments
// (GBRKC_GRID_MIN_NC overrides) and the engine's only one: such a system
// runs on every SM of the device as one grid team, where a cluster would
// give it 16 SMs.  GBRKC_GRID=0, or a forced cluster size
// (GBRKC_CLUSTER_SIZE), keeps it on a cluster.
bool grid_team_fits(const gbrkc_engine *E, const PoolHost &P) {
  const char *g = getenv("GBRKC_GRID");
  if (g && g[0] == '0') return false;
  const char *cs = getenv("GBRKC_CLUSTER_SIZE");
  if (cs && cs[0]) return false;
  const char *m = getenv("GBRKC_GRID_MIN_NC");
  const long min_nc = (m && m[0]) ? atol(m) : cluster_min_nc();
  if (P.systems.size() != 1 || P.max_nc < min_nc) return false;
  for (const HostSystem &S : E->systems)
    if (S.type != P.type) return false;
  return true;
}

// The grid team's shape for a system of nc compartments on at most cap
// co-resident CTAs: the threads per CTA (bw, a power of two from 32 to
// GRID_BLOCK, every one owning elements) and the CTA count.  It minimises the
// elements of the busiest CTA (every CTA integrates its elements' stages on
// its own SM's FP64 pipe), then the CTA count (every CTA takes part in every
// barrier); within the reduction's limits (at most GRID_MAX_BLOCKS chunks of
// bw elements, GRID_MAX_ROWS per thread).  GBRKC_GRID_BW and GBRKC_GRID_CTAS
// fix either.  Returns false when no shape fits.
bool grid_shape_rule(long nc, int cap, int want_bw, int want_ctas, int *bw_out, int *ctas_out) {
  long best_load = -1;
  for (int bw = 32; bw <= GRID_BLOCK; bw *= 2) {
    if (want_bw > 0 && bw != want_bw) continue;
    const long chunks = (nc + bw - 1) / bw;
    if (chunks > GRID_MAX_BLOCKS) continue;
    long ctas = std::min<long>(cap, chunks);
    if (want_ctas > 0) ctas = std::min<long>(cap, want_ctas);
    if (ctas < 1) continue;
    const long rows = (chunks + ctas - 1) / ctas;
    if (rows > GRID_MAX_ROWS) continue;
    const long load = rows * bw;
    if (best_load < 0 || load < best_load || (load == best_load && ctas < *ctas_out)) {
      best_load = load;
      *bw_out = bw;
      *ctas_out = (int)ctas;
    }
  }
  return best_load > 0;
}
bool grid_shape(long nc, int cap, int *bw_out, int *ctas_out) {
  const char *eb = getenv("GBRKC_GRID_BW"), *ec = getenv("GBRKC_GRID_CTAS");
  const int want_bw = (eb && eb[0]) ? atoi(eb) : 0, want_ctas = (ec && ec[0]) ? atoi(ec) : 0;
  return grid_shape_rule(nc, cap, want_bw, want_ctas, bw_out, ctas_out);
}

// Output compartments per cell: the voltage record (the soma; the
// reference's output_file columns) and the raster (the compartment whose
// threshold crossing output_file logs): gr.cu:257-280, go.cu:271-290,
// pkj.cu:371-390, io.cu:260-283.
int soma_comp(int type, int ncomp) {
  if (type == PKJ) return ncomp - 1;
  if (type == GO) return std::min(30, ncomp - 1);
  if (type == GR) return (ncomp == 578) ? 16 : std::min(1, ncomp - 1);
  return std::min(1, ncomp - 1);
}
int spike_comp(int type, int ncomp) {
  if (type == PKJ) return ncomp - 1;
  if (type == GO) return std::min(30, ncomp - 1);
  if (type == GR) return (ncomp == 578) ? 77 : ncomp - 1;
  return std::min(2, ncomp - 1);
}
double spike_threshold(int type) { return type == PKJ ? -10.0 : 10.0; }

// Controller state before initialisation (RKC_vec_initialize's h_others /
// h_work / h_bool, solve_rkc.cu:757-791): waiting for the init launch unless
// the system is a free slot; iv_left intervals may be advanced (-1: any).
Ctl initial_ctl(const HostSystem &S, int iv_left) {
  Ctl c{};
  for (int k = 0; k < 5; k++) c.map[k] = k;
  c.tend = H_MAX;
  c.last = 1; c.newspc = 1; c.jacatt = 0;
  c.tol = S.tol;
  c.hmin = S.hmin;
  c.integ = pow(2.0, log10(S.tol));
  c.status = S.idle ? 0 : ST_INIT;
  c.iv_left = S.idle ? 0 : iv_left;
  return c;
}

// System S's conductances (channel densities times its cells' scales), its
// initial state (*_initialize_ion: gr_ion.cu:635-672, go_ion.cu:590-634,
// pkj_ion.cu:360-395, io_ion.cu:163-194) and its stimulus, into the pool's
// host mirrors at compartment offset off and pool cell cell0.
void fill_state(gbrkc_engine *E, PoolHost &P, const HostSystem &S, long off, int cell0) {
  const int type = P.type, nion = NION[type], ncond = NCOND[type];
  const Template &T = E->templates[S.tmpl];
  const long nc = P.nc;
  for (int i = 0; i < S.nc; i++) {
    const int j = i % S.ncomp, cell = i / S.ncomp;
    const long g = off + i;
    if (!S.cond_scale_ch.empty()) {
      for (int k = 0; k < ncond; k++) P.cond[(size_t)k * nc + g] = T.cond[k][j] * S.cond_scale_ch[(size_t)cell * ncond + k];
    } else if (S.cond_scale.empty()) {
      for (int k = 0; k < ncond; k++) P.cond[(size_t)k * nc + g] = T.cond[k][j];
    } else {
      for (int k = 0; k < ncond; k++) P.cond[(size_t)k * nc + g] = T.cond[k][j] * S.cond_scale[cell];
    }
    CompInit ci;
    initial_state(type, S.jitter[cell], T.ctype[j], (type == IO) ? P.cond[(size_t)IO_g_CaH * nc + g] : 0.0, &ci);
    P.v[g] = ci.v; P.ca[g] = ci.ca; P.ca2[g] = ci.ca2; P.rev[g] = ci.rev; P.ca_old[g] = ci.ca_old;
    P.iext[g] = 0.0;
    for (int k = 0; k < nion; k++) P.ion[(size_t)k * nc + g] = ci.x[k];
  }
  for (int c = 0; c < S.n; c++) {
    P.stim_comp[cell0 + c] = S.stim_comp[c];
    P.stim_amp[cell0 + c] = S.stim_amp[c];
    P.stim_t0[cell0 + c] = S.stim_t0[c];
    P.stim_t1[cell0 + c] = S.stim_t1[c];
  }
}

int assemble_pool(gbrkc_engine *E, PoolHost &P) {
  const int type = P.type;
  const int nion = NION[type], ncond = NCOND[type];
  // count compartments
  long nc = 0;
  int ncell = 0;
  for (int id : P.systems) { nc += E->systems[id].nc; ncell += E->systems[id].n; }
  P.nc = nc;
  P.ncell = ncell;
  P.v.assign(nc, 0.0); P.ca.assign(nc, 0.0); P.ca2.assign(nc, 0.0); P.rev.assign(nc, 0.0);
  P.ca_old.assign(nc, 0.0); P.iext.assign(nc, 0.0); P.shell.assign(nc, 0.0); P.area.assign(nc, 0.0);
  P.ctype.assign(nc, 0); P.flags.assign(nc, 0);
  P.ion.assign((size_t)nion * nc, 0.0);
  P.cond.assign((size_t)ncond * nc, 0.0);
  long off = 0, ws = 0;
  int cell0 = 0;
  for (int id : P.systems) {
    HostSystem &S = E->systems[id];
    const Template &T = E->templates[S.tmpl];
    S.pool_index = (int)P.sys_off.size();
    P.sys_off.push_back((int)off);
    P.sys_nc.push_back(S.nc);
    P.sys_ncell.push_back(S.n);
    P.sys_ncomp.push_back(S.ncomp);
    P.sys_cell0.push_back(cell0);
    P.max_nc = std::max(P.max_nc, S.nc);
    P.min_nc = std::min(P.min_nc, S.nc);
    P.max_ncell = std::max(P.max_ncell, S.n);
    // template (pool-local)
    auto tl = P.tmpl_local.find(S.tmpl);
    if (tl == P.tmpl_local.end()) {
      int li = (int)P.t_row0.size();
      P.t_row0.push_back((int)P.t_row.size());
      P.t_nz0.push_back((int)P.t_col.size());
      P.t_cm0.push_back((int)P.t_invcm.size());
      // drop the diagonal (it multiplies y_i - y_i = 0); keep column order
      int cnt = 0;
      for (int r = 0; r < T.ncomp; r++) {
        P.t_row.push_back(cnt);
        double sum = 0.0;
        for (int j = T.row[r]; j < T.row[r + 1]; j++)
          if (T.col[j] != r) {
            P.t_col.push_back(T.col[j]);
            P.t_g.push_back(T.val[j]);
            P.t_gc.push_back(T.val[j] * T.invcm[r]);
            sum += T.val[j] * T.invcm[r];
            cnt++;
          }
        P.t_Gc.push_back(sum);
      }
      P.t_row.push_back(cnt);
      for (double x : T.invcm) P.t_invcm.push_back(x);
      tl = P.tmpl_local.emplace(S.tmpl, li).first;
    }
    P.sys_tmpl.push_back(tl->second);
    if (S.csr >= 0) {
      const SysCsr &C = E->csrs[S.csr];
      P.sys_csr.push_back((int)P.s_row0.size());
      P.s_row0.push_back((int)P.s_row.size());
      P.s_nz0.push_back((int)P.s_col.size());
      P.s_cm0.push_back((int)P.s_invcm.size());
      int cnt = 0;
      for (int r = 0; r < S.nc; r++) {
        P.s_row.push_back(cnt);
        double sum = 0.0;
        for (int j = C.row[r]; j < C.row[r + 1]; j++)
          if (C.col[j] != r) {
            P.s_col.push_back(C.col[j]);
            P.s_g.push_back(C.val[j]);
            P.s_gc.push_back(C.val[j] * C.invcm[r]);
            sum += C.val[j] * C.invcm[r];
            cnt++;
          }
        P.s_Gc.push_back(sum);
      }
      P.s_row.push_back(cnt);
      for (double x : C.invcm) P.s_invcm.push_back(x);
    } else {
      P.sys_csr.push_back(-1);
    }
    P.sys_gap0.push_back((int)P.gap_pre.size());
    P.sys_ngap.push_back((int)S.gap_pre.size());
    for (size_t e = 0; e < S.gap_pre.size(); e++) {
      P.gap_pre.push_back(S.gap_pre[e]);
      P.gap_post.push_back(S.gap_post[e]);
      P.gap_g.push_back(S.gap_g[e]);
    }
    P.sys_ws.push_back(ws);
    ws += (long)WS_VECS * ((S.nc + 1) & ~1);
    // per compartment static data, then the initial state
    for (int i = 0; i < S.nc; i++) {
      const int j = i % S.ncomp;
      const long g = off + i;
      P.ctype[g] = (uint8_t)T.ctype[j];
      P.area[g] = T.area[j];
      P.shell[g] = T.shell[j];
      if (type == PKJ && (i % 1599 == 0)) P.flags[g] |= 1;  // pkj_ion.cu:329
    }
    P.stim_comp.resize(cell0 + S.n);
    P.stim_amp.resize(cell0 + S.n);
    P.stim_t0.resize(cell0 + S.n);
    P.stim_t1.resize(cell0 + S.n);
    fill_state(E, P, S, off, cell0);
    for (int c = 0; c < S.n; c++) {
      P.cell_soma.push_back((int)(off + (long)c * S.ncomp + soma_comp(type, S.ncomp)));
      P.cell_spk.push_back((int)(off + (long)c * S.ncomp + spike_comp(type, S.ncomp)));
      P.cell_sys.push_back(id);
      P.cell_local.push_back(c);
    }
    P.ctl.push_back(initial_ctl(S, S.idle ? 0 : -1));
    off += S.nc;
    cell0 += S.n;
  }
  P.ws_total = ws;
  // launch configuration: team shape by system size, workspace in shared
  // memory when it fits
  // tiny cells: one system per thread, the block's first warps spread over
  // the SMs (a warp's FP64 instructions cost the same for 1 or 32 lanes, so
  // 32 systems side by side beat one system over 4 lanes)
  const int nsys = (int)P.systems.size();
  if (P.max_nc <= LANE_MAX_NC) {
    P.team = (P.type == GR && P.min_nc == 4 && P.max_nc == 4 && P.max_ncell == 1) ? TEAM_LANE4 : TEAM_THREAD;
    P.block = MEGA_BLOCK;
  }
  else if (P.max_nc <= 320) { P.team = TEAM_WARP; P.block = 128; }
  else if (grid_team_fits(E, P)) {
    // a lone large system: every SM of the device on it
    const int g = P.f64 ? grid_capacity<double>(P.type) : grid_capacity<float>(P.type);
    int bw = 0, ctas = 0;
    if (g > 0 && grid_shape(P.max_nc, g, &bw, &ctas)) {
      // CTAs of exactly the owning threads: every warp of a CTA repeats the
      // controller's scalar FP64 work, so a warp without elements only
      // costs FP64 issue slots
      P.team = TEAM_GRID;
      P.block = bw;
      P.grid = ctas;
      P.grid_bw = bw;
      P.ws_tile = (long)WS_VECS * ((P.max_nc + 1) & ~1);
      P.ws_in_smem = 0;
      // each CTA's operator rows in shared memory when they fit: row slots
      // of the widest row (diagonal dropped) of any of the pool's systems
      int maxdeg = 0;
      for (size_t k = 0; k < P.systems.size(); k++) {
        const bool own = P.sys_csr[k] >= 0;
        const int *r = own ? P.s_row.data() + P.s_row0[P.sys_csr[k]] : P.t_row.data() + P.t_row0[P.sys_tmpl[k]];
        const int nr = own ? P.sys_nc[k] : P.sys_ncomp[k];
        for (int j = 0; j < nr; j++) maxdeg = std::max(maxdeg, r[j + 1] - r[j]);
      }
      const long rl = (P.max_nc + (long)ctas * bw - 1) / ((long)ctas * bw) * bw;
      const bool fits = maxdeg > 0 && grid_rows_smem(rl, maxdeg) <= GRID_ROWS_SMEM_MAX;
      const char *ec = getenv("GBRKC_GRID_ROWS_SMEM");
      const bool want = !(ec && ec[0] == '0');
      P.grid_rl = (int)rl;
      P.grid_maxdeg = (fits && want) ? maxdeg : 0;
      P.smem = P.grid_maxdeg ? grid_rows_smem(rl, maxdeg) : 0;
      // each CTA's neighbours: the owners of its rows' columns and the CTAs
      // whose rows reach its elements (element i: CTA (i mod ctas*bw) / bw)
      P.grid_nbr.clear();
      const char *el = getenv("GBRKC_GRID_LOCAL");
      if (!(el && el[0] == '0')) {
        const long size = (long)ctas * bw;
        std::vector<std::vector<char>> adj(ctas, std::vector<char>(ctas, 0));
        for (size_t k = 0; k < P.systems.size(); k++) {
          const bool own = P.sys_csr[k] >= 0;
          const int nc = P.sys_nc[k], ncomp = P.sys_ncomp[k];
          const int *r = own ? P.s_row.data() + P.s_row0[P.sys_csr[k]] : P.t_row.data() + P.t_row0[P.sys_tmpl[k]];
          const int *cl = own ? P.s_col.data() + P.s_nz0[P.sys_csr[k]] : P.t_col.data() + P.t_nz0[P.sys_tmpl[k]];
          for (int i = 0; i < nc; i++) {
            const int j = (own || P.sys_ncell[k] == 1) ? i : i % ncomp, base = i - j;
            const int a = (int)((i % size) / bw);
            for (int e = r[j]; e < r[j + 1]; e++) {
              const int b = (int)(((base + cl[e]) % size) / bw);
              if (a != b) adj[a][b] = adj[b][a] = 1;
            }
          }
        }
        bool fit = true;
        std::vector<int> nb((size_t)ctas * (GRID_MAX_NBR + 1), 0);
        for (int a = 0; a < ctas && fit; a++) {
          int n = 0;
          for (int b = 0; b < ctas; b++)
            if (adj[a][b]) {
              if (n == GRID_MAX_NBR) { fit = false; break; }
              nb[(size_t)a * (GRID_MAX_NBR + 1) + 1 + n++] = b;
            }
          nb[(size_t)a * (GRID_MAX_NBR + 1)] = n;
        }
        if (fit) P.grid_nbr = std::move(nb);
      }
      return 0;
    }
    P.team = TEAM_CLUSTER16;
    P.block = 256;
  }
  else if (P.max_nc >= cluster_min_nc()) { P.team = TEAM_CLUSTER16; P.block = 256; }
  else { P.team = TEAM_BLOCK; P.block = 256; }
  if (P.team == TEAM_CLUSTER16) {
    // the workspace spread block-cyclically over the cluster's CTAs of 256
    // threads: 16 CTAs where the device co-schedules them (more FP64 pipes
    // per system), else 8; GBRKC_CLUSTER_SIZE=8 or 16 forces one
    const char *cs = getenv("GBRKC_CLUSTER_SIZE");
    const int forced = cs ? atoi(cs) : 0;
    for (int team : {TEAM_CLUSTER16, TEAM_CLUSTER8}) {
      const int C = team_cluster_size(team);
      if (forced && forced != C) continue;
      const long slot = (long)((((P.max_nc + 1) & ~1) + 256 * C - 1) / (256 * C)) * 256;
      const size_t need = ((size_t)WS_VECS * slot + CLUSTER_RED_DOUBLES) * sizeof(double);
      if (need > 200 * 1024 || slot / 256 > CLUSTER_MAX_ROWS) continue;
      const int cap = P.f64 ? cluster_capacity<double>(P.type, team, need)
                                                   : cluster_capacity<float>(P.type, team, need);
      if (cap < 1) continue;
      P.team = team;
      P.ws_tile = (long)WS_VECS * slot;
      P.ws_in_smem = 1;
      P.smem = need;
      P.grid = C * std::max(1, std::min(nsys, cap));
      return 0;
    }
    P.team = TEAM_BLOCK;  // too large to stage: one CTA with the workspace in HBM
  }
  const bool lanes = (P.team == TEAM_THREAD || P.team == TEAM_LANE4);
  // single-lane workspaces interleave across all MEGA_BLOCK threads of the
  // block, whichever of them hold a system
  const int teams = (P.team == TEAM_BLOCK) ? 1 : lanes ? MEGA_BLOCK : P.block / P.team;
  P.ws_tile = (long)WS_VECS * ((P.max_nc + 1) & ~1);
  const size_t need = (size_t)teams * P.ws_tile * sizeof(double);
  P.ws_in_smem = need <= 200 * 1024;
  if (lanes && !P.ws_in_smem) return fail(GBRKC_EINVAL, "single-lane pool workspace does not fit shared memory");
  P.smem = P.ws_in_smem ? need : 0;
  if (P.team == TEAM_THREAD || P.team == TEAM_LANE4) {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    P.grid = std::max(1, std::min((nsys + 31) / 32, sms));
  } else {
    P.grid = (nsys + teams - 1) / teams;
  }
  return 0;
}

template <typename R>
int upload_pool(gbrkc_engine *E, PoolHost &P, PoolView<R> &V) {
  DeviceMem &M = E->mem;
  int rc = 0;
  V.type = P.type;
  V.nsys = (int)P.systems.size();
  V.stride = P.nc;
#define UP(host, dev)                                    \
  do {                                                   \
    auto *tmp_ = (decltype(dev))nullptr;                 \
    using T_ = typename std::remove_const<typename std::remove_pointer<decltype(tmp_)>::type>::type; \
    T_ *d_ = nullptr;                                    \
    if ((rc = M.upload<T_>(host, &d_))) return rc;       \
    dev = d_;                                            \
  } while (0)
  UP(P.sys_off, V.sys_off); UP(P.sys_nc, V.sys_nc); UP(P.sys_ncell, V.sys_ncell);
  UP(P.sys_ncomp, V.sys_ncomp); UP(P.sys_tmpl, V.sys_tmpl); UP(P.sys_csr, V.sys_csr);
  UP(P.sys_cell0, V.sys_cell0); UP(P.sys_gap0, V.sys_gap0); UP(P.sys_ngap, V.sys_ngap);
  UP(P.sys_ws, V.sys_ws); UP(P.ctl, V.ctl);
  V.grid_red = nullptr;
  V.grid_bar = nullptr;
  V.grid_nbr = nullptr;
  V.grid_flags = nullptr;
  V.grid_bw = P.grid_bw;
  {
    // fence.acq_rel + acquire polls; GBRKC_GRID_FENCE=sc for __threadfence
    // on both sides of the wait (8% slower on the Purkinje 3x3 system)
    const char *f = getenv("GBRKC_GRID_FENCE");
    V.grid_light = (f && strcmp(f, "sc") == 0) ? 0 : 1;
  }
  V.grid_rl = P.grid_rl;
  V.grid_maxdeg = P.grid_maxdeg;
  if (P.team == TEAM_GRID) {
    const std::vector<double> red(2 * GRID_MAX_BLOCKS, 0.0);
    const std::vector<unsigned> bar(sizeof(GridBarrier) / sizeof(unsigned), 0u);
    UP(red, V.grid_red);
    UP(bar, V.grid_bar);
    P.d_grid_bar = V.grid_bar;
    if (!P.grid_nbr.empty()) {
      const std::vector<unsigned long long> fl((size_t)P.grid * 16, 0ull);
      UP(P.grid_nbr, V.grid_nbr);
      UP(fl, V.grid_flags);
      P.d_grid_flags = V.grid_flags;
    }
  }
  std::vector<double> zws(P.ws_total, 0.0);
  UP(zws, V.ws);
  std::vector<double> zero(P.nc, 0.0);
  UP(zero, V.ede); UP(zero, V.vnew);
  UP(P.v, V.v); UP(P.ca, V.ca); UP(P.ca2, V.ca2); UP(P.rev, V.rev); UP(P.ca_old, V.ca_old);
  UP(P.iext, V.iext); UP(P.shell, V.shell); UP(P.area, V.area);
  UP(P.ctype, V.ctype); UP(P.flags, V.flags);
  std::vector<R> ion(P.ion.begin(), P.ion.end()), cond(P.cond.begin(), P.cond.end());
  UP(ion, V.ion); UP(cond, V.cond);
  UP(P.t_row0, V.t_row0); UP(P.t_nz0, V.t_nz0); UP(P.t_cm0, V.t_cm0); UP(P.t_row, V.t_row);
  UP(P.t_col, V.t_col); UP(P.t_g, V.t_g); UP(P.t_invcm, V.t_invcm);
  UP(P.t_gc, V.t_gc); UP(P.t_Gc, V.t_Gc);
  UP(P.s_row0, V.s_row0); UP(P.s_nz0, V.s_nz0); UP(P.s_cm0, V.s_cm0); UP(P.s_row, V.s_row);
  UP(P.s_col, V.s_col); UP(P.s_g, V.s_g); UP(P.s_invcm, V.s_invcm);
  UP(P.s_gc, V.s_gc); UP(P.s_Gc, V.s_Gc);
  UP(P.gap_pre, V.gap_pre); UP(P.gap_post, V.gap_post); UP(P.gap_g, V.gap_g);
  UP(P.stim_comp, V.stim_comp); UP(P.stim_amp, V.stim_amp); UP(P.stim_t0, V.stim_t0);
  UP(P.stim_t1, V.stim_t1); UP(P.cell_soma, V.cell_soma); UP(P.cell_spk, V.cell_spk);
  std::vector<double> prev(P.ncell, 100.0);  // raster_prev starts at 100 (main.cu:163-169)
  UP(prev, V.spk_prev);
  std::vector<int> zc(1, 0);
  UP(zc, V.spk_count);
#undef UP
  V.spk_log = nullptr;
  V.spk_cap = 0;
  V.spk_th = spike_threshold(P.type);
  P.d_spk_prev = V.spk_prev;
  P.d_spk_count = V.spk_count;
  bool any_stim = false;
  for (int c : P.stim_comp) any_stim |= (c >= 0);
  V.stim_on = any_stim;
  V.coef = E->d_coef;
  V.coef_off = E->d_coef_off;
  V.coef_mmax = E->coef_mmax;
  // granule Na parameters per compartment type (gr_ion.cu:56-70)
  static const double n1[9] = {1, 1, 1, 1, 1, 5.422, 5.422, 5.422, 5.422};
  static const double n2[9] = {1, 1, 1, 1, 1, 3.279, 3.279, 3.279, 3.279};
  static const double n3[9] = {1, 1, 1, 1, 1, 1.83, 1.83, 1.83, 1.83};
  static const double n4[9] = {1, 1, 1, 1, 1, 0.738, 0.738, 0.738, 0.738};
  static const double Aa[9] = {1, 1, 1, 1, 1, 8.85, 8.85, 8.85, 8.85};
  static const double Ab[9] = {1, 1, 1, 1, 1, 0.0318, 0.0318, 0.0318, 0.0318};
  static const double Vs[9] = {1, 1, 1, 1, 1, -22.0, -22.0, -25.0, -25.0};
  static const double Con[9] = {1, 1, 1, 1, 1, 0.003464, 0.003464, 0.09353, 0.09353};
  static const double Coff[9] = {1, 1, 1, 1, 1, 0.4157, 0.4157, 0.04676, 0.04676};
  static const double Oon[9] = {1, 1, 1, 1, 1, 1.8186, 1.8186, 2.5981, 2.5981};
  static const double Ooff[9] = {1, 1, 1, 1, 1, 0.006928, 0.006928, 0.000173, 0.000173};
  for (int t = 0; t < 9; t++) {
    NaPar &p = V.na[t];
    p.n1 = n1[t]; p.n2 = n2[t]; p.n3 = n3[t]; p.n4 = n4[t]; p.Aa = Aa[t]; p.Ab = Ab[t]; p.vshift = Vs[t];
    p.Con = Con[t]; p.Coff = Coff[t]; p.Oon = Oon[t]; p.Ooff = Ooff[t];
    p.a = pow((Oon[t] / Con[t]), 0.25);
    p.b = pow((Ooff[t] / Coff[t]), 0.25);
    p.a4 = pow(p.a, 4.0);
    p.b4 = pow(p.b, 4.0);
  }
  V.soma_out = nullptr;
  V.lanes = E->lanes;
  V.rec_w = P.rec_w;
  P.d_cell_soma = const_cast<int *>(V.cell_soma);
  V.ncell_pool = P.ncell;
  V.ws_in_smem = P.ws_in_smem;
  V.ws_tile_doubles = P.ws_tile;
  P.d_ws = V.ws; P.d_vnew = V.vnew; P.d_v = V.v; P.d_ca = V.ca; P.d_rev = V.rev; P.d_ede = V.ede;
  P.d_ion = (void *)V.ion; P.d_ctl = V.ctl;
  return prepare_pool_kernel<R>(P.type, P.team, P.smem) ? fail(GBRKC_ECUDA, "cudaFuncSetAttribute failed") : 0;
}

// Launch every pool's kernel on its own stream (the pools run concurrently)
// and time the whole advance and each kernel with CUDA events recorded on the
// launching streams.
void rebalance_roles(gbrkc_engine *E, const double *role_ms, bool tune_gr);

template <typename R> PoolView<R> &pool_view(PoolHost &P);
template <> PoolView<double> &pool_view<double>(PoolHost &P) { return P.vd; }
template <> PoolView<float> &pool_view<float>(PoolHost &P) { return P.vf; }

// Whether the warps that give every granule system with work its own lane
// fit in half the CTAs the other roles leave (8 warps a CTA): then every
// system is in flight, the latency a request server needs; else lanes run
// several systems in turn and the role split decides the granule CTAs.
bool granules_all_in_flight(const gbrkc_engine *E, long warps) {
  int nother = 0;
  for (int t = 0; t < NTYPES; t++) nother += (t != GR && E->role_ctas[t] > 0);
  return (warps + MEGA_BLOCK / 32 - 1) / (MEGA_BLOCK / 32) <= (E->mega_grid - nother) / 2;
}

// Granule warps for the next persistent launch: one lane per granule system
// with work (parked slots, finished budgets and stopped systems need none).
// When they are all in flight (granules_all_in_flight) the granule CTAs are
// re-fitted to them at once, the other roles giving the difference; else
// the warps fill the granule role's CTAs (at most 8 a CTA) and lanes take
// further systems from the queue in turn (any count is correct).  CTAs the
// warps leave empty go to the other roles.
void fit_granule_warps(gbrkc_engine *E) {
  if (!E->mega || E->role_ctas[GR] == 0) return;
  PoolHost &G = E->pools[GR];
  const long active = (E->gr_active >= 0) ? E->gr_active : (long)G.systems.size();
  // the preferred lanes per warp, doubled while the warps would need more
  // than half of the CTAs' warp slots (the other roles need the rest)
  int lanes = E->lanes;
  while (lanes < 32 && (active + lanes - 1) / lanes > E->gr_warps_max / 2) lanes = std::min(32, 2 * lanes);
  G.vd.lanes = G.vf.lanes = lanes;
  const int per = MEGA_BLOCK / 32;
  const long need = std::max(1L, std::min((long)E->gr_warps_max, (active + lanes - 1) / lanes));
  E->gr_warps_need = (int)need;
  const bool all_in = granules_all_in_flight(E, need);
  const int want = all_in ? (int)need : (int)std::min(need, (long)per * E->role_ctas[GR]);
  E->gr_warps = want;
  const int c = all_in ? std::max((want + per - 1) / per, std::min(want, E->role_ctas[GR]))
                       : std::min(want, E->role_ctas[GR]);
  while (c > E->role_ctas[GR]) {  // take from the other role with the most CTAs
    int best = -1;
    for (int t = 0; t < NTYPES; t++)
      if (t != GR && E->role_ctas[t] > 1 && (best < 0 || E->role_ctas[t] > E->role_ctas[best])) best = t;
    if (best < 0) break;
    E->role_ctas[best]--;
    E->role_ctas[GR]++;
  }
  while (c < E->role_ctas[GR]) {  // give to the other role with the most work per CTA
    int best = -1;
    double bv = -1.0;
    for (int t = 0; t < NTYPES; t++) {
      if (t == GR || E->role_ctas[t] == 0 || E->role_ctas[t] >= E->role_cap[t]) continue;
      const double v = E->role_work[t] / E->role_ctas[t];
      if (v > bv) { bv = v; best = t; }
    }
    E->role_ctas[GR]--;
    if (best >= 0) E->role_ctas[best]++;
  }
}

// The persistent launch's pool views and role boundaries; returns the CTA
// count.
template <typename R>
int mega_pools(gbrkc_engine *E, MegaView<R> &M) {
  int end = 0;
  for (int t = 0; t < NTYPES; t++) {
    PoolHost &P = E->pools[t];
    M.pool[t] = P.systems.empty() ? PoolView<R>{} : pool_view<R>(P);
    end += E->role_ctas[t];
    M.role_end[t] = end;
  }
  return end;
}

template <typename R>
int launch_mega_all(gbrkc_engine *E, double t0, int n_iv, int iv0, int init) {
  MegaView<R> M{};
  const int end = mega_pools<R>(E, M);
  if (end > E->mega_grid || end <= 0)
    return fail(GBRKC_ESTATE, "persistent launch: %d role CTAs for a grid of %d", end, E->mega_grid);
  M.gr_nc4 = E->pools[GR].team == TEAM_LANE4;
  // granule warps spread as evenly as whole warps allow: the first
  // lane_extra CTAs take lane_warps + 1
  M.lane_warps = 0;
  M.lane_extra = 0;
  if (E->role_ctas[GR] > 0) {
    // the role split may have moved since the warps were fitted: at most 8
    // warps a CTA (lanes take further systems in turn)
    E->gr_warps = std::max(1, std::min(E->gr_warps, (MEGA_BLOCK / 32) * E->role_ctas[GR]));
    M.lane_warps = E->gr_warps / E->role_ctas[GR];
    M.lane_extra = E->gr_warps % E->role_ctas[GR];
    if (M.lane_warps + (M.lane_extra > 0) > MEGA_BLOCK / 32)
      return fail(GBRKC_ESTATE, "persistent launch: %d granule warps do not fit %d CTAs", E->gr_warps,
                  E->role_ctas[GR]);
  }
  if (E->role_ctas[GR] > 0 &&
      (!E->pools[GR].ws_in_smem ||
       E->mega_smem < (size_t)MEGA_BLOCK * (size_t)E->pools[GR].ws_tile * sizeof(double)))
    return fail(GBRKC_ESTATE, "persistent launch: granule workspaces do not fit its shared memory");
  M.queue = E->d_queue;
  M.t_start = E->d_tstart;
  M.t_end = E->d_tend;
  cudaStream_t st = E->streams[0];
  CUDA_TRY(cudaMemsetAsync(E->d_queue, 0, NTYPES * sizeof(int), st));
  CUDA_TRY(cudaEventRecord(E->ev_start, st));
  int rc = launch_mega<R>(M, end, E->mega_smem, st, t0, n_iv, iv0, init);
  if (rc) return fail(GBRKC_ECUDA, "persistent launch: %s", cudaGetErrorString((cudaError_t)rc));
  CUDA_TRY(cudaEventRecord(E->ev_end, st));
  CUDA_TRY(cudaEventSynchronize(E->ev_end));
  CUDA_TRY(cudaEventElapsedTime(&E->last_ms, E->ev_start, E->ev_end));
  // per-role makespans from the CTAs' device timestamps
  std::vector<unsigned long long> ts(end), te(end);
  CUDA_TRY(cudaMemcpy(ts.data(), E->d_tstart, end * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(te.data(), E->d_tend, end * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  unsigned long long t_first = ~0ull;
  for (int b = 0; b < end; b++) t_first = std::min(t_first, ts[b]);
  double role_ms[NTYPES] = {};
  int b = 0;
  for (int t = 0; t < NTYPES; t++) {
    unsigned long long last = t_first;
    for (int k = 0; k < E->role_ctas[t]; k++, b++) last = std::max(last, te[b]);
    role_ms[t] = E->role_ctas[t] ? (double)(last - t_first) * 1e-6 : 0.0;
    E->last_kernel_ms[t] = (float)role_ms[t];
  }
  if (!init && n_iv > 0) rebalance_roles(E, role_ms, true);
  return 0;
}

int launch_all(gbrkc_engine *E, double t0, int n_iv, int iv0, int init) {
  if (E->mega)
    return (E->precision == GBRKC_FP64) ? launch_mega_all<double>(E, t0, n_iv, iv0, init)
                                        : launch_mega_all<float>(E, t0, n_iv, iv0, init);
  CUDA_TRY(cudaEventRecord(E->ev_start, E->streams[0]));
  for (int t = 1; t < NTYPES; t++) CUDA_TRY(cudaStreamWaitEvent(E->streams[t], E->ev_start, 0));
  for (int t = 0; t < NTYPES; t++) {
    PoolHost &P = E->pools[t];
    if (P.systems.empty()) continue;
    int rc;
    if ((P.team == TEAM_THREAD || P.team == TEAM_LANE4) &&
        (P.block != MEGA_BLOCK || !P.ws_in_smem ||
         P.smem < (size_t)MEGA_BLOCK * (size_t)P.ws_tile * sizeof(double)))
      return fail(GBRKC_ESTATE, "single-lane pool %d: launch shape does not cover its workspaces", t);
    if (P.team == TEAM_GRID) {
      CUDA_TRY(cudaMemsetAsync(P.d_grid_bar, 0, sizeof(GridBarrier), E->streams[t]));
      if (P.d_grid_flags)
        CUDA_TRY(cudaMemsetAsync(P.d_grid_flags, 0, (size_t)P.grid * 16 * sizeof(unsigned long long), E->streams[t]));
    }
    CUDA_TRY(cudaEventRecord(E->ev_k0[t], E->streams[t]));
    if (P.f64)
      rc = launch_pool<double>(t, P.vd, P.team, P.grid, P.block, P.smem, E->streams[t], t0, n_iv, iv0, init);
    else
      rc = launch_pool<float>(t, P.vf, P.team, P.grid, P.block, P.smem, E->streams[t], t0, n_iv, iv0, init);
    if (rc) return fail(GBRKC_ECUDA, "launch (type %d): %s", t, cudaGetErrorString((cudaError_t)rc));
    CUDA_TRY(cudaEventRecord(E->ev_k1[t], E->streams[t]));
    if (t != 0) CUDA_TRY(cudaStreamWaitEvent(E->streams[0], E->ev_k1[t], 0));
  }
  CUDA_TRY(cudaEventRecord(E->ev_end, E->streams[0]));
  CUDA_TRY(cudaEventSynchronize(E->ev_end));
  for (int t = 0; t < NTYPES; t++) CUDA_TRY(cudaStreamSynchronize(E->streams[t]));
  CUDA_TRY(cudaEventElapsedTime(&E->last_ms, E->ev_start, E->ev_end));
  for (int t = 0; t < NTYPES; t++) {
    E->last_kernel_ms[t] = 0.0f;
    if (!E->pools[t].systems.empty()) CUDA_TRY(cudaEventElapsedTime(&E->last_kernel_ms[t], E->ev_k0[t], E->ev_k1[t]));
    if (E->pools[t].team == TEAM_GRID && !E->pools[t].systems.empty()) {
      GridBarrier gb{};
      CUDA_TRY(cudaMemcpy(&gb, E->pools[t].d_grid_bar, sizeof gb, cudaMemcpyDeviceToHost));
      if (gb.abort)
        return fail(GBRKC_ECUDA, "grid team (type %d): a barrier gave up waiting; the system is stopped", t);
    }
  }
  return 0;
}

int system_loc(gbrkc_engine *E, int id, PoolHost **P, HostSystem **S) {
  if (!E || id < 0 || id >= (int)E->systems.size()) return fail(GBRKC_EINVAL, "bad system id");
  if (!E->built) return fail(GBRKC_ESTATE, "engine not built");
  *S = &E->systems[id];
  *P = &E->pools[(*S)->type];
  return 0;
}

}  // namespace

namespace {

// Re-split the persistent launch's CTAs between roles so that they finish
// together.  Granule warps are latency-bound (a lone warp runs one dependent
// FP64 chain per system at ~64 cycles an operation): spreading them over more
// CTAs shortens their time only through less sharing of each SM's FP64 pipe,
// modelled as T ~ (warps per CTA)^0.5.  The other roles' time is taken as
// inversely proportional to the CTAs they get.  The granule CTA count moves
// halfway to where the two models cross; the other roles then split the
// remaining CTAs in proportion to their measured work (CTAs x makespan,
// smoothed over launches), each within its cap (a role cannot use more CTAs
// than it has teams of work).
void rebalance_roles(gbrkc_engine *E, const double *role_ms, bool tune_gr) {
  int avail = E->mega_grid;
  if (E->role_ctas[GR] > 0) {
    double others = 0.0;
    int nother = 0, other_ctas = 0;
    for (int t = 0; t < NTYPES; t++)
      if (t != GR && E->role_ctas[t] > 0) {
        others = std::max(others, role_ms[t]);
        nother++;
        other_ctas += E->role_ctas[t];
      }
    // granule role time on x CTAs, A warps giving every system a lane:
    // each lane runs max(1, A / 8x) systems in turn, and a system's serial
    // chain slows as sqrt(warps per CTA) (FP64 issue shared on the SM)
    const double A = std::max(1, E->gr_warps_need > 0 ? E->gr_warps_need : E->gr_warps);
    auto gr_time = [&](double x) {
      const double per = MEGA_BLOCK / 32;
      return sqrt(std::min(per, A / x)) * std::max(1.0, A / (per * x));
    };
    const int lo = granules_all_in_flight(E, (long)A)
                       ? std::max(1, std::min(E->mega_grid - nother, ((int)A + MEGA_BLOCK / 32 - 1) / (MEGA_BLOCK / 32)))
                       : 1;
    const int hi = std::max(lo, std::min((int)A, E->mega_grid - nother));
    int c = E->role_ctas[GR];
    if (tune_gr && others > 0.0 && role_ms[GR] > 0.0 && other_ctas > 0) {
      const double f0 = gr_time(c);
      int best = c;
      double bestv = 1e300;
      for (int x = lo; x <= hi; x++) {
        const double tg = role_ms[GR] * gr_time(x) / f0;
        const int oc = E->mega_grid - x;
        if (oc < nother) continue;
        const double to = others * (double)other_ctas / (double)oc;
        const double v = std::max(tg, to);
        if (v < bestv) { bestv = v; best = x; }
      }
      c = (c + best + 1) / 2;
    }
    E->role_ctas[GR] = std::max(lo, std::min(hi, c));
    avail -= E->role_ctas[GR];
  }
  // work per role (CTA-ms), smoothed over launches
  double work[NTYPES] = {}, total = 0.0;
  for (int t = 0; t < NTYPES; t++) {
    if (t == GR || E->role_ctas[t] == 0) continue;
    const double w = std::max(role_ms[t], 1e-3) * E->role_ctas[t];
    E->role_work[t] = (E->role_work[t] > 0.0) ? 0.5 * E->role_work[t] + 0.5 * w : w;
    work[t] = E->role_work[t];
    total += work[t];
  }
  if (total <= 0.0) return;
  int want[NTYPES] = {}, used = 0;
  for (int t = 0; t < NTYPES; t++) {
    if (t == GR || E->role_ctas[t] == 0) continue;
    const int n = (int)std::lround(avail * work[t] / total);
    want[t] = std::max(1, std::min(E->role_cap[t], n));
    used += want[t];
  }
  // fix the total by moving CTAs to / from the role with the largest work per CTA
  while (used != avail) {
    int best = -1;
    double bv = used < avail ? -1.0 : 1e300;
    for (int t = 0; t < NTYPES; t++) {
      if (t == GR || want[t] == 0) continue;
      const double v = work[t] / want[t];
      if (used < avail && want[t] < E->role_cap[t] && v > bv) { bv = v; best = t; }
      if (used > avail && want[t] > 1 && v < bv) { bv = v; best = t; }
    }
    if (best < 0) break;
    want[best] += used < avail ? 1 : -1;
    used += used < avail ? 1 : -1;
  }
  for (int t = 0; t < NTYPES; t++)
    if (t != GR) E->role_ctas[t] = want[t];
}

// Decide whether all pools fit the persistent launch's team shapes and size
// its shared memory; sets each pool's team / workspace placement.
int setup_mega(gbrkc_engine *E) {
  const char *no = getenv("GBRKC_NO_MEGA");
  if (no && no[0] == '1') return 0;
  // a mixed engine with FP64 granule pools advances each type in its own
  // launch (the granule pool's FP64 kernel beside the others' FP32 kernels,
  // on their own streams): the persistent kernel holds one precision
  if (E->gr_f64 && !E->pools[GR].systems.empty()) return 0;
  // pools of very large systems run on clusters, one launch per pool
  for (int t = 0; t < NTYPES; t++)
    if (!E->pools[t].systems.empty() &&
        (team_cluster_size(E->pools[t].team) > 0 || E->pools[t].team == TEAM_GRID)) return 0;
  const PoolHost &G = E->pools[GR], &O = E->pools[GO];
  if (!G.systems.empty() && G.max_nc > LANE_MAX_NC) return 0;
  if (!O.systems.empty() && O.max_nc > 320) return 0;
  // granule CTAs run up to MEGA_BLOCK single-lane systems (capped below at one
  // warp per CTA); Golgi 8 warps; Purkinje / olive one system per CTA
  const int teams[NTYPES] = {32, MEGA_BLOCK / TEAM_WARP, 1, 1};
  const int team_kind[NTYPES] = {(G.min_nc == 4 && G.max_nc == 4 && G.max_ncell == 1) ? TEAM_LANE4 : TEAM_THREAD, TEAM_WARP,
                                 TEAM_BLOCK, TEAM_BLOCK};
  size_t smem = 0;
  int nonempty = 0;
  for (int t = 0; t < NTYPES; t++) {
    PoolHost &P = E->pools[t];
    if (P.systems.empty()) continue;
    nonempty++;
    P.team = team_kind[t];
    P.block = MEGA_BLOCK;
    P.ws_tile = (long)WS_VECS * ((P.max_nc + 1) & ~1);
    const size_t need = (size_t)(t == GR ? MEGA_BLOCK : teams[t]) * P.ws_tile * sizeof(double);
    P.ws_in_smem = need <= 200 * 1024;
    if (t == GR && !P.ws_in_smem) return 0;
    if (P.ws_in_smem) smem = std::max(smem, need);
    const int nsys = (int)P.systems.size();
    E->role_cap[t] = (nsys + teams[t] - 1) / teams[t];
  }
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int bps = 0;
  int rc = (E->precision == GBRKC_FP64) ? prepare_mega_kernel<double>(smem, &bps) : prepare_mega_kernel<float>(smem, &bps);
  if (rc || bps <= 0) return 0;
  E->mega_grid = sms * bps;
  if (E->mega_grid < nonempty) return 0;
  E->mega_smem = smem;
  E->mega = true;
  // first split: granule warps two to a CTA (or spread over every CTA when
  // granules are alone); the rest by compartment count with per-type weights;
  // refined after every launch
  // lanes take further systems from the queue, so the warps never need to
  // exceed what the CTAs left after one per other role can hold
  {
    int others_n = 0;
    for (int t = 1; t < NTYPES; t++) others_n += !E->pools[t].systems.empty();
    E->gr_warps_max = (E->mega_grid - others_n) * (MEGA_BLOCK / 32);
    const long need = ((long)E->pools[GR].systems.size() + 31) / 32;
    E->gr_warps = (int)std::min<long>(need, E->gr_warps_max);
    E->gr_warps_need = E->gr_warps;
  }
  const double w[NTYPES] = {0.0, 1.0, 0.35, 3.0};
  double ms[NTYPES];
  int others = 0;
  for (int t = 0; t < NTYPES; t++) {
    PoolHost &P = E->pools[t];
    E->role_ctas[t] = P.systems.empty() ? 0 : 1;
    ms[t] = P.systems.empty() ? 0.0 : w[t] * (double)P.nc;
    others += (t != GR && !P.systems.empty());
  }
  if (E->role_ctas[GR] > 0) {
    // two granule warps to a CTA beside other roles, else spread over all;
    // beside other roles at most the granule share of the estimated work (a
    // granule compartment costs about 29 Golgi compartments: the granule
    // controller's tolerance of 1e-9 keeps its steps short)
    E->role_ctas[GR] = others ? (E->gr_warps + 1) / 2 : std::min(E->gr_warps, E->mega_grid);
    if (others) {
      double wo = 0.0;
      for (int t = 1; t < NTYPES; t++) wo += w[t] * (double)E->pools[t].nc;
      const double wg = 29.0 * (double)E->pools[GR].nc;
      E->role_ctas[GR] = std::min(E->role_ctas[GR], std::max(1, (int)(E->mega_grid * wg / (wg + wo))));
    }
    E->role_ctas[GR] = std::max(1, std::min(E->role_ctas[GR], E->mega_grid - others));
  }
  rebalance_roles(E, ms, false);
  // the first launch's granule warps fit the granule CTAs (lanes take
  // further systems in turn)
  E->gr_warps = std::min(E->gr_warps, (MEGA_BLOCK / 32) * E->role_ctas[GR]);
  for (int t = 0; t < NTYPES; t++) E->role_work[t] = 0.0;
  return 0;
}

}  // namespace

namespace {

// Resolve every synapse to pool compartments, index the synapses of each
// pool by post compartment in (kind, id) order, and upload the tables.
int build_synapses(gbrkc_engine *E) {
  const int n = (int)E->syn.kind.size();
  if (n == 0) return 0;
  // reversal potentials, syn.cuh:13,20,31,38 (E_MFGR, E_GRGO, E_GOGR, E_GRPKJ)
  static const double E_KIND[SYN_KINDS] = {0.0, 0.0, -82.0, 0.0};
  // decay per state, exp(-RKC_DT / tau): syn.cuh:14-15, 21-23, 32-33, 40
  static const double TAU[8] = {1.2, 52.0, 1.5, 31.0, 170.0, 7.0, 59.0, 6.0};
  std::vector<int> pre_type(n, -1), post_type(n);
  std::vector<long> pre_gi(n, 0), post_gi(n);
  std::vector<double> e(n), zero(n, 0.0), old_v(n, 1000.0);  // old_v starts at 1000 (syn.cu:176,330,510)
  for (int i = 0; i < n; i++) {
    const HostSystem &Q = E->systems[E->syn.post_sys[i]];
    post_type[i] = Q.type;
    post_gi[i] = E->pools[Q.type].sys_off[Q.pool_index] + E->syn.post_comp[i];
    if (E->syn.kind[i] != SYN_MFGR) {
      const HostSystem &S = E->systems[E->syn.pre_sys[i]];
      pre_type[i] = S.type;
      pre_gi[i] = E->pools[S.type].sys_off[S.pool_index] + E->syn.pre_comp[i];
    }
    e[i] = E_KIND[E->syn.kind[i]];
  }
  DeviceMem &M = E->mem;
  int rc = 0;
  double *d_e = nullptr, *d_val = nullptr;
  SynView &V = E->sv;
  V.n = n;
  {
    int *p;
    if ((rc = M.upload(E->syn.kind, &p))) return rc;
    V.kind = p;
    if ((rc = M.upload(E->syn.grp, &p))) return rc;
    V.grp = p;
    if ((rc = M.upload(pre_type, &p))) return rc;
    V.pre_type = p;
    long *q;
    if ((rc = M.upload(pre_gi, &q))) return rc;
    V.pre_gi = q;
    double *d;
    if ((rc = M.upload(E->syn.w, &d))) return rc;
    V.w = d;
    if ((rc = M.upload(zero, &V.s0))) return rc;
    if ((rc = M.upload(zero, &V.s1))) return rc;
    if ((rc = M.upload(zero, &V.s2))) return rc;
    if ((rc = M.upload(zero, &d_val))) return rc;
    V.val = d_val;
    if ((rc = M.upload(old_v, &V.old_v))) return rc;
    if ((rc = M.upload(e, &d_e))) return rc;
    if ((rc = M.upload(E->syn.grp_rate, &d))) return rc;
    V.grp_rate = d;
    unsigned long long *u;
    if ((rc = M.upload(E->syn.grp_seed, &u))) return rc;
    V.grp_seed = u;
    V.ring = nullptr;
    V.delay = nullptr;
    bool any_delay = false;
    for (unsigned char x : E->syn.delay) any_delay |= (x != 0);
    if (any_delay) {
      std::vector<unsigned long long> ring(n, 0ull);
      if ((rc = M.upload(ring, &V.ring))) return rc;
      unsigned char *dl;
      if ((rc = M.upload(E->syn.delay, &dl))) return rc;
      V.delay = dl;
    }
  }
  for (int k = 0; k < 8; k++) V.decay[k] = exp(-0.125 / TAU[k]);
  for (int t = 0; t < NTYPES; t++) V.pre_v[t] = E->pools[t].d_v;
  // per pool: CSR over post compartments
  for (int t = 0; t < NTYPES; t++) {
    PoolHost &P = E->pools[t];
    if (P.systems.empty()) continue;
    std::vector<int> ids;
    for (int i = 0; i < n; i++)
      if (post_type[i] == t) ids.push_back(i);
    if (ids.empty()) continue;
    std::stable_sort(ids.begin(), ids.end(), [&](int a, int b) {
      if (post_gi[a] != post_gi[b]) return post_gi[a] < post_gi[b];
      if (E->syn.kind[a] != E->syn.kind[b]) return E->syn.kind[a] < E->syn.kind[b];
      return a < b;
    });
    std::vector<int> row(P.nc + 1, 0);
    for (int i : ids) row[post_gi[i] + 1]++;
    for (long c = 0; c < P.nc; c++) row[c + 1] += row[c];
    std::vector<double> buf(P.nc, 0.0);
    int *d_row = nullptr, *d_idx = nullptr;
    double *d_buf = nullptr;
    if ((rc = M.upload(row, &d_row))) return rc;
    if ((rc = M.upload(ids, &d_idx))) return rc;
    if ((rc = M.upload(buf, &d_buf))) return rc;
    const int mode = (t == GR) ? SYN_AT_ION : (t == GO) ? SYN_BUFFERED : (t == PKJ) ? SYN_BUFFERED_DECAY : SYN_NONE;
    if (mode == SYN_NONE) return fail(GBRKC_EINVAL, "synapses onto pool %d are not supported", t);
    P.vd.syn_mode = P.vf.syn_mode = mode;
    P.vd.syn_row = P.vf.syn_row = d_row;
    P.vd.syn_idx = P.vf.syn_idx = d_idx;
    P.vd.syn_val = P.vf.syn_val = d_val;
    P.vd.syn_e = P.vf.syn_e = d_e;
    P.vd.syn_buf = P.vf.syn_buf = d_buf;
  }
  return 0;
}

}  // namespace

static int add_synapses_impl(gbrkc_engine *E, const gbrkc_synapse_desc *d, int *first_id) {
  if (!E || !d) return fail(GBRKC_EINVAL, "null argument");
  if (E->built) return fail(GBRKC_ESTATE, "synapses must be added before gbrkc_build");
  if (d->kind < 0 || d->kind >= SYN_KINDS) return fail(GBRKC_EINVAL, "bad synapse kind %d", d->kind);
  if (d->n < 0) return fail(GBRKC_EINVAL, "bad synapse count");
  if (d->n > 0 && (!d->post_system || !d->post_comp || !d->weight)) return fail(GBRKC_EINVAL, "missing arrays");
  const bool poisson = d->kind == SYN_MFGR;
  if (d->n > 0 && !poisson && (!d->pre_system || !d->pre_comp)) return fail(GBRKC_EINVAL, "missing presynaptic arrays");
  // expected (pre, post) cell types per kind
  static const int PRE[SYN_KINDS] = {-1, GR, GO, GR}, POST[SYN_KINDS] = {GR, GO, GR, PKJ};
  const int nsys = (int)E->systems.size();
  for (int i = 0; i < d->n; i++) {
    if (d->delay && (d->delay[i] < 0 || d->delay[i] > 63))
      return fail(GBRKC_EINVAL, "synapse %d: delay %d outside 0..63 intervals", i, d->delay[i]);
    const int q = d->post_system[i];
    if (q < 0 || q >= nsys || E->systems[q].type != POST[d->kind] || d->post_comp[i] < 0 ||
        d->post_comp[i] >= E->systems[q].nc)
      return fail(GBRKC_EINVAL, "synapse %d: bad postsynaptic system or compartment", i);
    if (!poisson) {
      const int p = d->pre_system[i];
      if (p < 0 || p >= nsys || E->systems[p].type != PRE[d->kind] || d->pre_comp[i] < 0 ||
          d->pre_comp[i] >= E->systems[p].nc)
        return fail(GBRKC_EINVAL, "synapse %d: bad presynaptic system or compartment", i);
    }
  }
  const int grp = (int)E->syn.grp_seed.size();
  if (first_id) *first_id = (int)E->syn.kind.size();
  for (int i = 0; i < d->n; i++) {
    E->syn.kind.push_back(d->kind);
    E->syn.grp.push_back(grp);
    E->syn.pre_sys.push_back(poisson ? -1 : d->pre_system[i]);
    E->syn.pre_comp.push_back(poisson ? 0 : d->pre_comp[i]);
    E->syn.post_sys.push_back(d->post_system[i]);
    E->syn.post_comp.push_back(d->post_comp[i]);
    E->syn.w.push_back(d->weight[i]);
    E->syn.delay.push_back(d->delay ? (unsigned char)d->delay[i] : 0);
  }
  // mossy-fibre rates: 5 Hz, 60 Hz for S_Stimuli <= t < E_Stimuli (syn.cu:93-95,
  // param.h:8-9) unless the group gives its own
  const bool deflt = d->rate_base == 0.0 && d->rate_stim == 0.0 && d->stim_t0 == 0.0 && d->stim_t1 == 0.0;
  E->syn.grp_rate.push_back(deflt ? 5.0 : d->rate_base);
  E->syn.grp_rate.push_back(deflt ? 60.0 : d->rate_stim);
  E->syn.grp_rate.push_back(deflt ? 900.0 : d->stim_t0);
  E->syn.grp_rate.push_back(deflt ? 1000.0 : d->stim_t1);
  E->syn.grp_seed.push_back(d->seed);
  return 0;
}

extern "C" int gbrkc_add_synapses(gbrkc_engine *E, const gbrkc_synapse_desc *d, int *first_id) {
  return no_throw([&] { return add_synapses_impl(E, d, first_id); });
}

extern "C" int gbrkc_read_synapses(gbrkc_engine *E, int field, double *host, long n) {
  if (!E || !host) return fail(GBRKC_EINVAL, "null argument");
  if (!E->built) return fail(GBRKC_ESTATE, "engine not built");
  if (n < 0 || n > E->sv.n) return fail(GBRKC_EINVAL, "bad count");
  const double *src = nullptr;
  switch (field) {
    case GBRKC_SYNF_VAL: src = E->sv.val; break;
    case GBRKC_SYNF_S0: src = E->sv.s0; break;
    case GBRKC_SYNF_S1: src = E->sv.s1; break;
    case GBRKC_SYNF_S2: src = E->sv.s2; break;
    case GBRKC_SYNF_OLD_V: src = E->sv.old_v; break;
    default: return fail(GBRKC_EINVAL, "bad synapse field");
  }
  if (n == 0) return 0;
  CUDA_TRY(cudaMemcpy(host, src, n * sizeof(double), cudaMemcpyDeviceToHost));
  return 0;
}

static int build_impl(gbrkc_engine *E) {
  if (!E) return fail(GBRKC_EINVAL, "null engine");
  if (E->built) return fail(GBRKC_ESTATE, "already built");
  if (E->systems.empty()) return fail(GBRKC_EINVAL, "no systems");
  E->coef_mmax = 1024;
  coef_table(E->coef_mmax, E->coef, E->coef_off);
  {
    int rc = E->mem.upload(E->coef, &E->d_coef);
    if (rc) return rc;
    rc = E->mem.upload(E->coef_off, &E->d_coef_off);
    if (rc) return rc;
  }
  for (int t = 0; t < NTYPES; t++) { E->pools[t] = PoolHost(); E->pools[t].type = t; }
  for (int id = 0; id < (int)E->systems.size(); id++) E->pools[E->systems[id].type].systems.push_back(id);
  for (int t = 0; t < NTYPES; t++) {
    PoolHost &P = E->pools[t];
    if (P.systems.empty()) continue;
    P.f64 = E->precision == GBRKC_FP64 || (t == GR && E->gr_f64);
    int rc = assemble_pool(E, P);
    if (rc) return rc;
  }
  {
    int rc = setup_mega(E);
    if (rc) return rc;
  }
  for (int t = 0; t < NTYPES; t++) {
    PoolHost &P = E->pools[t];
    if (P.systems.empty()) continue;
    int rc = P.f64 ? upload_pool<double>(E, P, P.vd) : upload_pool<float>(E, P, P.vf);
    if (rc) return rc;
  }
  if (E->mega) {
    std::vector<int> q(NTYPES, 0);
    std::vector<unsigned long long> z(E->mega_grid, 0ull);
    int rc = E->mem.upload(q, &E->d_queue);
    if (!rc) rc = E->mem.upload(z, &E->d_tstart);
    if (!rc) rc = E->mem.upload(z, &E->d_tend);
    if (rc) return rc;
    // gbrkc_advance_noalloc's scratch: its address is taken here, while the
    // engine's device is current, so that the advance itself only reads it
    // (and an engine built after a device reset gets the new module's address)
    rc = noalloc_scratch(&E->d_static_scratch);
    if (rc) return fail(GBRKC_ECUDA, "static scratch: %s", cudaGetErrorString((cudaError_t)rc));
  }
  {
    int rc = build_synapses(E);
    if (rc) return rc;
  }
  E->built = true;
  int rc = launch_all(E, 0.0, 0, 0, 1);
  if (rc) { E->built = false; return rc; }
  return 0;
}

extern "C" int gbrkc_build(gbrkc_engine *E) { return no_throw([&] { return build_impl(E); }); }

extern "C" int gbrkc_advance(gbrkc_engine *E, double t0, int n_iv) {
  if (!E || n_iv < 0) return fail(GBRKC_EINVAL, "bad arguments");
  if (!E->built) return fail(GBRKC_ESTATE, "engine not built");
  int iv0 = E->soma_iv;
  for (int t = 0; t < NTYPES; t++) {
    PoolHost &P = E->pools[t];
    double *so = (E->soma_cap > 0 && iv0 + n_iv <= E->soma_cap) ? P.d_soma : nullptr;
    P.vd.soma_out = so;
    P.vf.soma_out = so;
  }
  int rc = 0;
  fit_granule_warps(E);
  if (E->pending_init) {
    // systems reset since the last call: initialise them (only them) first
    rc = launch_all(E, t0, 0, iv0, 1);
    if (rc) return rc;
    E->pending_init = false;
  }
  if (E->sv.n > 0) {
    // network mode: every system advances one interval, then the synapses
    // update from the new presynaptic voltages (main.cu:196-305)
    for (int k = 0; k < n_iv && !rc; k++) {
      rc = launch_all(E, t0 + k * H_MAX, 1, iv0 + k, 0);
      if (rc) break;
      rc = launch_syn_update(E->sv, E->streams[0], t0 + k * H_MAX, E->syn_interval++);
      if (rc) return fail(GBRKC_ECUDA, "synapse update: %s", cudaGetErrorString((cudaError_t)rc));
      CUDA_TRY(cudaStreamSynchronize(E->streams[0]));
    }
  } else {
    rc = launch_all(E, t0, n_iv, iv0, 0);
  }
  if (rc) return rc;
  if (E->soma_cap > 0) E->soma_iv += n_iv;
  // A system that stops (non-finite step, loop bound) is retired: it keeps
  // its last state, the kernels skip it from now on, and every other system
  // goes on.  The call reports systems that stopped during it.
  int newly = 0, first_id = -1, first_status = 0;
  for (int t = 0; t < NTYPES; t++) {
    PoolHost &P = E->pools[t];
    if (P.systems.empty()) continue;
    std::vector<Ctl> c(P.systems.size());
    CUDA_TRY(cudaMemcpy(c.data(), P.d_ctl, c.size() * sizeof(Ctl), cudaMemcpyDeviceToHost));
    if (P.retired.size() != c.size()) P.retired.assign(c.size(), 0);
    if (t == GR) {
      long active = 0;
      for (const Ctl &x : c) active += (x.status == 0 && x.iv_left != 0);
      E->gr_active = active;
    }
    for (size_t i = 0; i < c.size(); i++)
      if (c[i].status && !P.retired[i]) {
        P.retired[i] = 1;
        E->n_retired++;
        if (!newly++) { first_id = P.systems[i]; first_status = c[i].status; }
      }
  }
  if (newly)
    return fail(GBRKC_ESOLVER, "%d system(s) stopped (first: system %d, status %d); the others advanced", newly,
                first_id, first_status);
  return 0;
}

extern "C" int gbrkc_retired_systems(gbrkc_engine *E) { return E ? E->n_retired : 0; }

// ------------------------------------------------------- gbrkc_autotune
// Granule systems run one per lane; how many lanes of a warp take systems
// (cells per warp, hence per CTA) trades divergence -- a warp runs the union
// of its lanes' step-attempt paths -- against warps, i.e. CTAs taken from the
// other roles.  The best count depends on the workload's dynamics and mix,
// so it is measured: the same launch (t0, n_iv, from the engine's present
// state) runs once per candidate, twice each, from a device snapshot of the
// engine, and the fastest candidate is kept.  Scheduling never changes a
// system's arithmetic, so every candidate computes the same bits; the state,
// the CTA split between roles and the soma / spike records are restored
// afterwards, so the call leaves the simulation where it found it.
namespace {

struct Snapshot {
  std::vector<void *> dev;
  std::vector<std::pair<void *, size_t>> src;
  ~Snapshot() {
    for (void *p : dev) cudaFree(p);
  }
  int take(void *p, size_t n) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, n);
    if (e != cudaSuccess) return fail(GBRKC_ENOMEM, "autotune snapshot: %s", cudaGetErrorString(e));
    dev.push_back(q);
    src.push_back({p, n});
    e = cudaMemcpy(q, p, n, cudaMemcpyDeviceToDevice);
    if (e != cudaSuccess) return fail(GBRKC_ECUDA, "autotune snapshot: %s", cudaGetErrorString(e));
    return 0;
  }
  int restore() const {
    for (size_t k = 0; k < dev.size(); k++) {
      cudaError_t e = cudaMemcpy(src[k].first, dev[k], src[k].second, cudaMemcpyDeviceToDevice);
      if (e != cudaSuccess) return fail(GBRKC_ECUDA, "autotune restore: %s", cudaGetErrorString(e));
    }
    return 0;
  }
};

int autotune_impl(gbrkc_engine *E, double t0, int n_iv, int *lanes_out) {
  if (!E || n_iv <= 0 || !lanes_out) return fail(GBRKC_EINVAL, "bad arguments");
  if (!E->built) return fail(GBRKC_ESTATE, "engine not built");
  if (E->sv.n > 0) return fail(GBRKC_EINVAL, "engines with synapses are not tuned");
  *lanes_out = E->lanes;
  if (!E->mega || E->role_ctas[GR] == 0) return 0;      // no granule lanes to tune
  int rc;
  if (E->pending_init) {
    // systems reset since the last advance: initialise them first, as the
    // next advance would
    if ((rc = launch_all(E, t0, 0, E->soma_iv, 1))) return rc;
    E->pending_init = false;
  }
  Snapshot S;
  for (size_t k = 0; k < E->mem.ptrs.size(); k++)
    if ((rc = S.take(E->mem.ptrs[k], E->mem.sizes[k]))) return rc;
  for (auto &P : E->pools)
    if (P.d_spk_log && P.spk_cap > 0 && (rc = S.take(P.d_spk_log, (size_t)P.spk_cap * sizeof(SpikeRec)))) return rc;
  int ctas[NTYPES], warps = E->gr_warps, warps_need = E->gr_warps_need, lanes0 = E->lanes;
  double work[NTYPES];
  for (int t = 0; t < NTYPES; t++) { ctas[t] = E->role_ctas[t]; work[t] = E->role_work[t]; }
  const long active = E->gr_active;
  auto restore_host = [&]() {
    for (int t = 0; t < NTYPES; t++) { E->role_ctas[t] = ctas[t]; E->role_work[t] = work[t]; }
    E->gr_warps = warps;
    E->gr_warps_need = warps_need;
    E->gr_active = active;
  };
  for (int t = 0; t < NTYPES; t++) {
    E->pools[t].vd.soma_out = nullptr;     // the records are not written while tuning
    E->pools[t].vf.soma_out = nullptr;
  }
  static const int cand[] = {32, 16, 8};
  int best = lanes0;
  double best_ms = 1e300;
  for (int c : cand) {
    for (int rep = 0; rep < 2; rep++) {
      if ((rc = S.restore())) return rc;
      restore_host();
      E->lanes = c;
      fit_granule_warps(E);
      if ((rc = launch_all(E, t0, n_iv, E->soma_iv, 0))) return rc;
      if (E->last_ms < best_ms) { best_ms = E->last_ms; best = c; }
    }
  }
  if ((rc = S.restore())) return rc;
  restore_host();
  E->lanes = best;
  *lanes_out = best;
  return 0;
}

}  // namespace

extern "C" int gbrkc_autotune(gbrkc_engine *E, double t0, int n_iv, int *lanes_out) {
  return no_throw([&] { return autotune_impl(E, t0, n_iv, lanes_out); });
}

extern "C" int gbrkc_read(gbrkc_engine *E, int id, int field, int k, double *host, long n) {
  PoolHost *P = nullptr;
  HostSystem *S = nullptr;
  int rc = system_loc(E, id, &P, &S);
  if (rc) return rc;
  if (!host || n < 0 || n > S->nc) return fail(GBRKC_EINVAL, "bad buffer");
  const long off = P->sys_off[S->pool_index];
  const double *src = nullptr;
  switch (field) {
    case GBRKC_F_VNEW: src = P->d_vnew; break;
    case GBRKC_F_V: src = P->d_v; break;
    case GBRKC_F_CA: src = P->d_ca; break;
    case GBRKC_F_REV: src = P->d_rev; break;
    case GBRKC_F_B:
    case GBRKC_F_YN: {
      Ctl c;
      CUDA_TRY(cudaMemcpy(&c, P->d_ctl + S->pool_index, sizeof c, cudaMemcpyDeviceToHost));
      const long ncp = (S->nc + 1) & ~1;
      const long slot = (field == GBRKC_F_B) ? WS_B : c.map[1];
      CUDA_TRY(cudaMemcpy(host, P->d_ws + P->sys_ws[S->pool_index] + slot * ncp, n * sizeof(double), cudaMemcpyDeviceToHost));
      return 0;
    }
    case GBRKC_F_ION: {
      if (k < 0 || k >= NION[S->type]) return fail(GBRKC_EINVAL, "bad ion slot");
      if (P->f64) {
        CUDA_TRY(cudaMemcpy(host, (double *)P->d_ion + (size_t)k * P->nc + off, n * sizeof(double), cudaMemcpyDeviceToHost));
      } else {
        std::vector<float> tmp(n);
        CUDA_TRY(cudaMemcpy(tmp.data(), (float *)P->d_ion + (size_t)k * P->nc + off, n * sizeof(float), cudaMemcpyDeviceToHost));
        for (long i = 0; i < n; i++) host[i] = tmp[i];
      }
      return 0;
    }
    default: return fail(GBRKC_EINVAL, "bad field");
  }
  CUDA_TRY(cudaMemcpy(host, src + off, n * sizeof(double), cudaMemcpyDeviceToHost));
  return 0;
}

extern "C" int gbrkc_field_device_ptr(gbrkc_engine *E, int id, int field, double **ptr) {
  PoolHost *P = nullptr;
  HostSystem *S = nullptr;
  int rc = system_loc(E, id, &P, &S);
  if (rc) return rc;
  if (!ptr) return fail(GBRKC_EINVAL, "null output");
  const long off = P->sys_off[S->pool_index];
  double *base = nullptr;
  switch (field) {
    case GBRKC_F_VNEW: base = P->d_vnew; break;
    case GBRKC_F_V: base = P->d_v; break;
    case GBRKC_F_CA: base = P->d_ca; break;
    case GBRKC_F_REV: base = P->d_rev; break;
    case GBRKC_F_IEXT: base = P->f64 ? P->vd.iext : P->vf.iext; break;
    default: return fail(GBRKC_EINVAL, "field %d has no per-compartment device array", field);
  }
  *ptr = base ? base + off : nullptr;
  return 0;
}

extern "C" int gbrkc_system_ctl(gbrkc_engine *E, int id, double *ctl8, long long *stats6, int *status) {
  PoolHost *P = nullptr;
  HostSystem *S = nullptr;
  int rc = system_loc(E, id, &P, &S);
  if (rc) return rc;
  Ctl c;
  CUDA_TRY(cudaMemcpy(&c, P->d_ctl + S->pool_index, sizeof c, cudaMemcpyDeviceToHost));
  if (ctl8) {
    ctl8[0] = c.absh; ctl8[1] = c.sprad; ctl8[2] = c.naccpt; ctl8[3] = c.errold;
    ctl8[4] = c.hold; ctl8[5] = c.lt; ctl8[6] = c.tend; ctl8[7] = c.sum_dt;
  }
  if (stats6) {
    stats6[0] = c.n_steps; stats6[1] = c.n_rej; stats6[2] = c.n_stage; stats6[3] = c.n_rho;
    stats6[4] = c.n_ion; stats6[5] = c.n_rho_iter;
  }
  if (status) *status = c.status;
  return 0;
}

extern "C" int gbrkc_set_stim(gbrkc_engine *E, int id, const int *comp, const double *amp,
                              const double *t0, const double *t1) {
  PoolHost *P = nullptr;
  HostSystem *S = nullptr;
  int rc = system_loc(E, id, &P, &S);
  if (rc) return rc;
  if (!comp || !amp || !t0 || !t1) return fail(GBRKC_EINVAL, "null stimulus");
  for (int c = 0; c < S->n; c++)
    if (comp[c] >= S->ncomp) return fail(GBRKC_EINVAL, "stimulus compartment out of range");
  const int c0 = P->sys_cell0[S->pool_index];
  const bool f64 = P->f64;
  int *dc = const_cast<int *>(f64 ? P->vd.stim_comp : P->vf.stim_comp);
  double *da = const_cast<double *>(f64 ? P->vd.stim_amp : P->vf.stim_amp);
  double *d0 = const_cast<double *>(f64 ? P->vd.stim_t0 : P->vf.stim_t0);
  double *d1 = const_cast<double *>(f64 ? P->vd.stim_t1 : P->vf.stim_t1);
  cudaStream_t st = E->streams[S->type];
  CUDA_TRY(cudaMemcpyAsync(dc + c0, comp, S->n * sizeof(int), cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(da + c0, amp, S->n * sizeof(double), cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(d0 + c0, t0, S->n * sizeof(double), cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(d1 + c0, t1, S->n * sizeof(double), cudaMemcpyHostToDevice, st));
  P->vd.stim_on = 1;
  P->vf.stim_on = 1;
  CUDA_TRY(cudaStreamSynchronize(st));
  return 0;
}

extern "C" int gbrkc_type_cells(gbrkc_engine *E, int type) {
  if (!E || type < 0 || type >= NTYPES) return fail(GBRKC_EINVAL, "bad type");
  int n = 0;
  for (auto &s : E->systems)
    if (s.type == type) n += s.n;
  return n;
}

extern "C" int gbrkc_set_stim_type(gbrkc_engine *E, int type, const int *comp, const double *amp,
                                   const double *t0, const double *t1) {
  if (!E || type < 0 || type >= NTYPES || !comp || !amp || !t0 || !t1) return fail(GBRKC_EINVAL, "bad arguments");
  if (!E->built) return fail(GBRKC_ESTATE, "engine not built");
  PoolHost &P = E->pools[type];
  if (P.systems.empty()) return 0;
  // validate against each cell's own compartment count
  int cell = 0;
  for (int id : P.systems) {
    const HostSystem &S = E->systems[id];
    for (int c = 0; c < S.n; c++, cell++)
      if (comp[cell] >= S.ncomp) return fail(GBRKC_EINVAL, "stimulus compartment out of range");
  }
  const bool f64 = P.f64;
  int *dc = const_cast<int *>(f64 ? P.vd.stim_comp : P.vf.stim_comp);
  double *da = const_cast<double *>(f64 ? P.vd.stim_amp : P.vf.stim_amp);
  double *d0 = const_cast<double *>(f64 ? P.vd.stim_t0 : P.vf.stim_t0);
  double *d1 = const_cast<double *>(f64 ? P.vd.stim_t1 : P.vf.stim_t1);
  cudaStream_t st = E->streams[type];
  CUDA_TRY(cudaMemcpyAsync(dc, comp, P.ncell * sizeof(int), cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(da, amp, P.ncell * sizeof(double), cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(d0, t0, P.ncell * sizeof(double), cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(d1, t1, P.ncell * sizeof(double), cudaMemcpyHostToDevice, st));
  P.vd.stim_on = 1;
  P.vf.stim_on = 1;
  return 0;
}

extern "C" int gbrkc_read_soma_type(gbrkc_engine *E, int type, int n_iv, double *host) {
  if (!E || type < 0 || type >= NTYPES || !host) return fail(GBRKC_EINVAL, "bad arguments");
  PoolHost &P = E->pools[type];
  if (P.systems.empty()) return 0;
  if (!P.d_soma || n_iv < 0 || n_iv > E->soma_iv) return fail(GBRKC_EINVAL, "no such recording");
  CUDA_TRY(cudaMemcpyAsync(host, P.d_soma, (size_t)n_iv * P.ncell * P.rec_w * sizeof(double), cudaMemcpyDeviceToHost,
                           E->streams[type]));
  CUDA_TRY(cudaStreamSynchronize(E->streams[type]));
  return 0;
}

extern "C" int gbrkc_rewind_soma(gbrkc_engine *E) {
  if (!E) return fail(GBRKC_EINVAL, "null engine");
  E->soma_iv = 0;
  return 0;
}

// sum over systems of (stage evaluations + step attempts) x compartments:
// the compartment-update count of the benchmark metric
extern "C" long long gbrkc_compartment_updates(gbrkc_engine *E, int type) {
  if (!E || !E->built) return (long long)fail(GBRKC_ESTATE, "engine not built");
  long long total = 0;
  for (int t = 0; t < NTYPES; t++) {
    if (type >= 0 && t != type) continue;
    PoolHost &P = E->pools[t];
    if (P.systems.empty()) continue;
    std::vector<Ctl> c(P.systems.size());
    if (cudaMemcpy(c.data(), P.d_ctl, c.size() * sizeof(Ctl), cudaMemcpyDeviceToHost) != cudaSuccess)
      return (long long)fail(GBRKC_ECUDA, "reading counters failed");
    for (size_t i = 0; i < c.size(); i++) total += (c[i].n_stage + c[i].n_steps) * (long long)P.sys_nc[i];
  }
  return total;
}

extern "C" float gbrkc_last_advance_ms(gbrkc_engine *E) { return E ? E->last_ms : 0.0f; }

extern "C" int gbrkc_launch_layout(gbrkc_engine *E, int *ctas_per_type) {
  if (!E || !E->built) return fail(GBRKC_ESTATE, "engine not built");
  for (int t = 0; t < NTYPES; t++)
    ctas_per_type[t] = E->mega ? E->role_ctas[t] : E->pools[t].systems.empty() ? 0 : E->pools[t].grid;
  return E->mega ? 1 : 0;
}
extern "C" int gbrkc_grid_shape(long long nc, int max_ctas, int *threads_per_cta, int *ctas) {
  if (nc <= 0 || max_ctas <= 0 || !threads_per_cta || !ctas) return fail(GBRKC_EINVAL, "bad arguments");
  int bw = 0, n = 0;
  if (!grid_shape_rule((long)nc, max_ctas, 0, 0, &bw, &n))
    return fail(GBRKC_EINVAL, "no grid-team shape holds %lld compartments", nc);
  *threads_per_cta = bw;
  *ctas = n;
  return 0;
}
extern "C" int gbrkc_type_team(gbrkc_engine *E, int type) {
  if (!E || type < 0 || type >= NTYPES) return fail(GBRKC_EINVAL, "bad arguments");
  if (!E->built) return fail(GBRKC_ESTATE, "engine not built");
  const PoolHost &P = E->pools[type];
  if (P.systems.empty()) return 0;
  if (E->mega) return GBRKC_TEAM_MEGA;
  if (P.team == TEAM_GRID) return GBRKC_TEAM_GRID;
  if (team_cluster_size(P.team) > 0) return GBRKC_TEAM_CLUSTER;
  return GBRKC_TEAM_POOL;
}
extern "C" float gbrkc_last_kernel_ms(gbrkc_engine *E, int type) {
  return (E && type >= 0 && type < NTYPES) ? E->last_kernel_ms[type] : 0.0f;
}

extern "C" int gbrkc_system_nc(gbrkc_engine *E, int id) {
  if (!E || id < 0 || id >= (int)E->systems.size()) return fail(GBRKC_EINVAL, "bad system id");
  return E->systems[id].nc;
}

extern "C" long gbrkc_total_compartments(gbrkc_engine *E) {
  if (!E) return 0;
  long n = 0;
  for (auto &s : E->systems) n += s.nc;
  return n;
}

static int record_soma_impl(gbrkc_engine *E, int n_max) {
  if (!E || n_max < 0) return fail(GBRKC_EINVAL, "bad arguments");
  if (!E->built) return fail(GBRKC_ESTATE, "engine not built");
  E->soma_cap = n_max;
  E->soma_iv = 0;
  for (int t = 0; t < NTYPES; t++) {
    PoolHost &P = E->pools[t];
    if (P.systems.empty() || n_max == 0) { P.d_soma = nullptr; continue; }
    std::vector<double> z((size_t)n_max * P.ncell * P.rec_w, 0.0);
    int rc = E->mem.upload(z, &P.d_soma);
    if (rc) return rc;
  }
  return 0;
}

extern "C" int gbrkc_record_soma(gbrkc_engine *E, int n_max) {
  return no_throw([&] { return record_soma_impl(E, n_max); });
}

extern "C" int gbrkc_record_width(gbrkc_engine *E, int type, int width) {
  if (!E || type < 0 || type >= NTYPES || width < 1) return fail(GBRKC_EINVAL, "bad arguments");
  if (!E->built) return fail(GBRKC_ESTATE, "engine not built");
  PoolHost &P = E->pools[type];
  if (P.systems.empty()) return 0;
  if (E->soma_cap > 0) return fail(GBRKC_ESTATE, "set the width before gbrkc_record_soma");
  std::vector<int> first(P.ncell);
  for (size_t k = 0; k < P.systems.size(); k++) {
    const HostSystem &S = E->systems[P.systems[k]];
    if (width > S.ncomp) return fail(GBRKC_EINVAL, "width %d exceeds a cell's %d compartments", width, S.ncomp);
    for (int c = 0; c < S.n; c++) {
      const long base = P.sys_off[k] + (long)c * S.ncomp;
      first[P.sys_cell0[k] + c] = (int)(width == 1 ? base + soma_comp(type, S.ncomp) : base);
    }
  }
  CUDA_TRY(cudaMemcpy(P.d_cell_soma, first.data(), first.size() * sizeof(int), cudaMemcpyHostToDevice));
  P.cell_soma = first;
  P.rec_w = width;
  P.vd.rec_w = P.vf.rec_w = width;
  return 0;
}

static int read_soma_impl(gbrkc_engine *E, int id, int n_iv, double *host) {
  PoolHost *P = nullptr;
  HostSystem *S = nullptr;
  int rc = system_loc(E, id, &P, &S);
  if (rc) return rc;
  if (!P->d_soma || n_iv < 0 || n_iv > E->soma_iv || !host) return fail(GBRKC_EINVAL, "no such recording");
  const int c0 = P->sys_cell0[S->pool_index], w = P->rec_w;
  std::vector<double> all((size_t)n_iv * P->ncell * w);
  CUDA_TRY(cudaMemcpy(all.data(), P->d_soma, all.size() * sizeof(double), cudaMemcpyDeviceToHost));
  for (int k = 0; k < n_iv; k++)
    for (int c = 0; c < S->n * w; c++)
      host[(size_t)k * S->n * w + c] = all[((size_t)k * P->ncell + c0) * w + c];
  return 0;
}

extern "C" int gbrkc_read_soma(gbrkc_engine *E, int id, int n_iv, double *host) {
  return no_throw([&] { return read_soma_impl(E, id, n_iv, host); });
}

// ------------------------------------------------------- slots and raster
namespace {

// Systems first_id .. first_id + n - 1 as one run of one pool (consecutive
// pool positions): their pool and first position, or an error.
int system_run(gbrkc_engine *E, int first_id, int n, PoolHost **Pout, int *pi0) {
  if (!E || n <= 0 || first_id < 0 || first_id + (long)n > (long)E->systems.size())
    return fail(GBRKC_EINVAL, "bad system range");
  if (!E->built) return fail(GBRKC_ESTATE, "engine not built");
  const int type = E->systems[first_id].type;
  PoolHost &P = E->pools[type];
  const int p0 = E->systems[first_id].pool_index;
  for (int k = 1; k < n; k++) {
    const HostSystem &S = E->systems[first_id + k];
    if (S.type != type || S.pool_index != p0 + k)
      return fail(GBRKC_EINVAL, "systems %d..%d are not one run of one cell type", first_id, first_id + n - 1);
  }
  *Pout = &P;
  *pi0 = p0;
  return 0;
}

// Copy the host mirrors of pool positions pi0 .. pi1 - 1 (their compartments,
// cells, edges, workspaces and controllers) to the device, with the
// workspace, ede and v_new cleared as at build.
template <typename R>
int upload_run(gbrkc_engine *E, PoolHost &P, int pi0, int pi1) {
  PoolView<R> &V = pool_view<R>(P);
  cudaStream_t st = E->streams[0];
  const long o0 = P.sys_off[pi0], o1 = (long)P.sys_off[pi1 - 1] + P.sys_nc[pi1 - 1];
  const long nco = o1 - o0, nc = P.nc;
  const int c0 = P.sys_cell0[pi0], c1 = P.sys_cell0[pi1 - 1] + P.sys_ncell[pi1 - 1];
  const long w0 = P.sys_ws[pi0], w1 = P.sys_ws[pi1 - 1] + (long)WS_VECS * ((P.sys_nc[pi1 - 1] + 1) & ~1);
  auto put = [&](void *dev, const void *host, size_t bytes) -> int {
    CUDA_TRY(cudaMemcpyAsync(dev, host, bytes, cudaMemcpyHostToDevice, st));
    return 0;
  };
  int rc = 0;
  const size_t db = nco * sizeof(double);
  if ((rc = put(V.v + o0, P.v.data() + o0, db)) || (rc = put(V.ca + o0, P.ca.data() + o0, db)) ||
      (rc = put(V.ca2 + o0, P.ca2.data() + o0, db)) || (rc = put(V.rev + o0, P.rev.data() + o0, db)) ||
      (rc = put(V.ca_old + o0, P.ca_old.data() + o0, db)) || (rc = put(V.iext + o0, P.iext.data() + o0, db)))
    return rc;
  const int nion = NION[P.type], ncond = NCOND[P.type];
  std::vector<R> tmp((size_t)(nion + ncond) * nco);
  for (int k = 0; k < nion; k++)
    for (long i = 0; i < nco; i++) tmp[(size_t)k * nco + i] = (R)P.ion[(size_t)k * nc + o0 + i];
  for (int k = 0; k < ncond; k++)
    for (long i = 0; i < nco; i++) tmp[(size_t)(nion + k) * nco + i] = (R)P.cond[(size_t)k * nc + o0 + i];
  for (int k = 0; k < nion; k++)
    if ((rc = put(V.ion + (size_t)k * nc + o0, tmp.data() + (size_t)k * nco, nco * sizeof(R)))) return rc;
  for (int k = 0; k < ncond; k++)
    if ((rc = put(const_cast<R *>(V.cond) + (size_t)k * nc + o0, tmp.data() + (size_t)(nion + k) * nco,
                  nco * sizeof(R))))
      return rc;
  CUDA_TRY(cudaMemsetAsync(V.ws + w0, 0, (w1 - w0) * sizeof(double), st));
  CUDA_TRY(cudaMemsetAsync(V.ede + o0, 0, db, st));
  CUDA_TRY(cudaMemsetAsync(V.vnew + o0, 0, db, st));
  const size_t nce = c1 - c0;
  std::vector<double> prev(nce, 100.0);
  if ((rc = put(const_cast<int *>(V.stim_comp) + c0, P.stim_comp.data() + c0, nce * sizeof(int))) ||
      (rc = put(const_cast<double *>(V.stim_amp) + c0, P.stim_amp.data() + c0, nce * sizeof(double))) ||
      (rc = put(const_cast<double *>(V.stim_t0) + c0, P.stim_t0.data() + c0, nce * sizeof(double))) ||
      (rc = put(const_cast<double *>(V.stim_t1) + c0, P.stim_t1.data() + c0, nce * sizeof(double))) ||
      (rc = put(V.spk_prev + c0, prev.data(), nce * sizeof(double))))
    return rc;
  const int g0 = P.sys_gap0[pi0], g1 = P.sys_gap0[pi1 - 1] + P.sys_ngap[pi1 - 1];
  if (g1 > g0 && (rc = put(const_cast<double *>(V.gap_g) + g0, P.gap_g.data() + g0, (g1 - g0) * sizeof(double))))
    return rc;
  if ((rc = put(V.ctl + pi0, P.ctl.data() + pi0, (pi1 - pi0) * sizeof(Ctl)))) return rc;
  CUDA_TRY(cudaStreamSynchronize(st));
  bool any_stim = false;
  for (int c : P.stim_comp) any_stim |= (c >= 0);
  P.vd.stim_on = any_stim;
  P.vf.stim_on = any_stim;
  return 0;
}

}  // namespace

static int systems_reset_impl(gbrkc_engine *E, int first_id, int n, const gbrkc_reset_desc *d) {
  PoolHost *P = nullptr;
  int pi0 = 0;
  int rc = system_run(E, first_id, n, &P, &pi0);
  if (rc) return rc;
  if (!d || !d->jitter) return fail(GBRKC_EINVAL, "null argument");
  if (d->n_intervals < -1) return fail(GBRKC_EINVAL, "interval budget must be >= -1");
  if (E->sv.n > 0) return fail(GBRKC_EINVAL, "engines with synapses cannot reset systems");
  if (d->stim_comp && (!d->stim_amp || !d->stim_t0 || !d->stim_t1)) return fail(GBRKC_EINVAL, "incomplete stimulus");
  // validate everything before changing anything
  long cells = 0, edges = 0;
  std::vector<std::vector<double>> new_gap_g(n);  // the olive systems' new edge conductances
  for (int k = 0; k < n; k++) {
    const HostSystem &S = E->systems[first_id + k];
    for (int c = 0; c < S.n; c++) {
      if (d->stim_comp && d->stim_comp[cells + c] >= S.ncomp)
        return fail(GBRKC_EINVAL, "stimulus compartment out of range");
      if (d->cond_scale) {
        const double x = d->cond_scale[cells + c];
        if (!(x >= 0.0) || !std::isfinite(x)) return fail(GBRKC_EINVAL, "conductance scale must be finite and >= 0");
      }
      if (d->cond_scale_ch)
        for (int q = 0; q < NCOND[S.type]; q++) {
          const double x = d->cond_scale_ch[(size_t)(cells + c) * NCOND[S.type] + q];
          if (!(x >= 0.0) || !std::isfinite(x)) return fail(GBRKC_EINVAL, "conductance scale must be finite and >= 0");
        }
    }
    if (d->io_gap_g && S.type == IO && !S.gap_pre.empty()) {
      // same edges, new conductances (gap.cu:4-120)
      HostSystem G = S;
      G.io_gap_g.assign(d->io_gap_g + 4 * cells, d->io_gap_g + 4 * (cells + S.n));
      G.gap_pre.clear(); G.gap_post.clear(); G.gap_g.clear();
      if ((rc = build_io_gap(G))) return rc;
      if (G.gap_pre != S.gap_pre || G.gap_post != S.gap_post)
        return fail(GBRKC_EINVAL, "io_gap_g changes the edge set of system %d (a conductance of 0?)", first_id + k);
      new_gap_g[k] = std::move(G.gap_g);
      edges += 4L * S.n;
    }
    cells += S.n;
  }
  if (d->io_gap_g && edges == 0) return fail(GBRKC_EINVAL, "io_gap_g given for systems without IO gap junctions");
  cells = 0;
  for (int k = 0; k < n; k++) {
    HostSystem &S = E->systems[first_id + k];
    const int pi = pi0 + k;
    S.idle = false;
    S.jitter.assign(d->jitter + cells, d->jitter + cells + S.n);
    for (int c = 0; c < S.n; c++) {
      const bool on = d->stim_comp && d->stim_comp[cells + c] >= 0;
      S.stim_comp[c] = on ? d->stim_comp[cells + c] : -1;
      S.stim_amp[c] = on ? d->stim_amp[cells + c] : 0.0;
      S.stim_t0[c] = on ? d->stim_t0[cells + c] : 0.0;
      S.stim_t1[c] = on ? d->stim_t1[cells + c] : 0.0;
    }
    if (d->cond_scale) S.cond_scale.assign(d->cond_scale + cells, d->cond_scale + cells + S.n);
    else S.cond_scale.clear();
    if (d->cond_scale_ch)
      S.cond_scale_ch.assign(d->cond_scale_ch + (size_t)cells * NCOND[S.type],
                             d->cond_scale_ch + (size_t)(cells + S.n) * NCOND[S.type]);
    else S.cond_scale_ch.clear();
    if (d->io_gap_g && S.type == IO && !S.gap_pre.empty()) {
      S.io_gap_g.assign(d->io_gap_g + 4 * cells, d->io_gap_g + 4 * (cells + S.n));
      S.gap_g = std::move(new_gap_g[k]);
      std::copy(S.gap_g.begin(), S.gap_g.end(), P->gap_g.begin() + P->sys_gap0[pi]);
    }
    fill_state(E, *P, S, P->sys_off[pi], P->sys_cell0[pi]);
    P->ctl[pi] = initial_ctl(S, d->n_intervals);
    if ((int)P->retired.size() > pi) P->retired[pi] = 0;
    cells += S.n;
  }
  rc = P->f64 ? upload_run<double>(E, *P, pi0, pi0 + n) : upload_run<float>(E, *P, pi0, pi0 + n);
  if (rc) return rc;
  E->pending_init = true;
  if (P->type == GR && E->gr_active >= 0) E->gr_active += n;
  return 0;
}

extern "C" int gbrkc_systems_reset(gbrkc_engine *E, int first_id, int n, const gbrkc_reset_desc *d) {
  return no_throw([&] { return systems_reset_impl(E, first_id, n, d); });
}

extern "C" int gbrkc_read_run(gbrkc_engine *E, int first_id, int n, int field, double *host, long cap) {
  PoolHost *P = nullptr;
  int pi0 = 0;
  int rc = system_run(E, first_id, n, &P, &pi0);
  if (rc) return rc;
  const long o0 = P->sys_off[pi0], o1 = (long)P->sys_off[pi0 + n - 1] + P->sys_nc[pi0 + n - 1];
  if (!host || cap < o1 - o0) return fail(GBRKC_EINVAL, "buffer holds %ld of %ld values", cap, o1 - o0);
  const double *src = nullptr;
  switch (field) {
    case GBRKC_F_VNEW: src = P->d_vnew; break;
    case GBRKC_F_V: src = P->d_v; break;
    case GBRKC_F_CA: src = P->d_ca; break;
    case GBRKC_F_REV: src = P->d_rev; break;
    default: return fail(GBRKC_EINVAL, "field not readable by runs");
  }
  CUDA_TRY(cudaMemcpy(host, src + o0, (o1 - o0) * sizeof(double), cudaMemcpyDeviceToHost));
  return 0;
}

extern "C" int gbrkc_run_status(gbrkc_engine *E, int first_id, int n, int *status, int *iv_left) {
  PoolHost *P = nullptr;
  int pi0 = 0;
  int rc = system_run(E, first_id, n, &P, &pi0);
  if (rc) return rc;
  if (status)
    CUDA_TRY(cudaMemcpy2D(status, sizeof(int), (const char *)(P->d_ctl + pi0) + offsetof(Ctl, status), sizeof(Ctl),
                          sizeof(int), n, cudaMemcpyDeviceToHost));
  if (iv_left)
    CUDA_TRY(cudaMemcpy2D(iv_left, sizeof(int), (const char *)(P->d_ctl + pi0) + offsetof(Ctl, iv_left), sizeof(Ctl),
                          sizeof(int), n, cudaMemcpyDeviceToHost));
  return 0;
}

extern "C" int gbrkc_set_budget(gbrkc_engine *E, int first_id, int n, int n_intervals) {
  PoolHost *P = nullptr;
  int pi0 = 0;
  int rc = system_run(E, first_id, n, &P, &pi0);
  if (rc) return rc;
  if (n_intervals < -1) return fail(GBRKC_EINVAL, "interval budget must be >= -1");
  std::vector<int> v(n, n_intervals);
  CUDA_TRY(cudaMemcpy2D((char *)(P->d_ctl + pi0) + offsetof(Ctl, iv_left), sizeof(Ctl), v.data(), sizeof(int),
                        sizeof(int), n, cudaMemcpyHostToDevice));
  for (int k = 0; k < n; k++) P->ctl[pi0 + k].iv_left = n_intervals;
  return 0;
}

static int record_spikes_impl(gbrkc_engine *E, long capacity) {
  if (!E || capacity < 0 || capacity > (1L << 30)) return fail(GBRKC_EINVAL, "bad arguments");
  if (!E->built) return fail(GBRKC_ESTATE, "engine not built");
  for (int t = 0; t < NTYPES; t++) {
    PoolHost &P = E->pools[t];
    if (P.systems.empty()) continue;
    if (P.d_spk_log) CUDA_TRY(cudaFree(P.d_spk_log));
    P.d_spk_log = nullptr;
    P.spk_cap = 0;
    if (capacity > 0) {
      cudaError_t e = cudaMalloc((void **)&P.d_spk_log, capacity * sizeof(SpikeRec));
      if (e != cudaSuccess) return fail(GBRKC_ENOMEM, "spike log: %s", cudaGetErrorString(e));
      P.spk_cap = (int)capacity;
    }
    CUDA_TRY(cudaMemset(P.d_spk_count, 0, sizeof(int)));
    P.vd.spk_log = P.vf.spk_log = P.d_spk_log;
    P.vd.spk_cap = P.vf.spk_cap = P.spk_cap;
  }
  return 0;
}

extern "C" int gbrkc_record_spikes(gbrkc_engine *E, long capacity) {
  return no_throw([&] { return record_spikes_impl(E, capacity); });
}

static int read_spikes_impl(gbrkc_engine *E, int type, long cap, double *t, int *sys, int *cell, long *n) {
  if (!E || type < 0 || type >= NTYPES || cap < 0 || !n || (cap > 0 && (!t || !sys || !cell)))
    return fail(GBRKC_EINVAL, "bad arguments");
  if (!E->built) return fail(GBRKC_ESTATE, "engine not built");
  *n = 0;
  PoolHost &P = E->pools[type];
  if (P.systems.empty() || !P.d_spk_log) return 0;
  int cnt = 0;
  CUDA_TRY(cudaMemcpy(&cnt, P.d_spk_count, sizeof(int), cudaMemcpyDeviceToHost));
  const long avail = std::min<long>(cnt, P.spk_cap);
  std::vector<SpikeRec> r(avail);
  if (avail > 0) CUDA_TRY(cudaMemcpy(r.data(), P.d_spk_log, avail * sizeof(SpikeRec), cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemset(P.d_spk_count, 0, sizeof(int)));
  // the device appends in completion order: sort by time, then pool cell
  std::sort(r.begin(), r.end(), [](const SpikeRec &a, const SpikeRec &b) {
    return a.t < b.t || (a.t == b.t && a.cell < b.cell);
  });
  const long m = std::min(avail, cap);
  for (long k = 0; k < m; k++) {
    t[k] = r[k].t;
    sys[k] = P.cell_sys[r[k].cell];
    cell[k] = P.cell_local[r[k].cell];
  }
  *n = m;
  if (cnt > P.spk_cap || avail > cap)
    return fail(GBRKC_EOVERFLOW, "%ld spike(s) lost (logged %d, log capacity %d, read capacity %ld)",
                (long)cnt - m, cnt, P.spk_cap, cap);
  return 0;
}

extern "C" int gbrkc_read_spikes(gbrkc_engine *E, int type, long cap, double *t, int *sys, int *cell, long *n) {
  return no_throw([&] { return read_spikes_impl(E, type, cap, t, sys, cell, n); });
}

extern "C" long gbrkc_rkc_coefficients(int m, double *out, long cap) {
  if (m < 1 || m > 1024 || cap < 0 || (!out && cap > 0)) return fail(GBRKC_EINVAL, "bad arguments");
  std::vector<double> coef;
  std::vector<long> off;
  coef_table(m, coef, off);
  const long n = off[m + 1] - off[m];
  if (cap < n) return fail(GBRKC_EINVAL, "buffer holds %ld of %ld values", cap, n);
  std::copy(coef.begin() + off[m], coef.begin() + off[m + 1], out);
  return n;
}

extern "C" long long gbrkc_system_bytes(int precision, int cell_type, int ncomp, int ncell) {
  if (cell_type < 0 || cell_type >= NTYPES || ncomp <= 0 || ncell <= 0) return fail(GBRKC_EINVAL, "bad shape");
  const long long nc = (long long)ncomp * ncell;
  const long long rb = (precision == GBRKC_FP64 || (cell_type == GR && mixed_granules_fp64())) ? 8 : 4;
  long long b = nc * (WS_VECS * 8 + 10 * 8 + 2 + rb * (NION[cell_type] + NCOND[cell_type]));
  b += (long long)ncell * (3 * 4 + 4 * 8 + 2 * 4);          // stimulus, output maps, raster
  b += 12 * 4 + 8 + (long long)sizeof(Ctl);                  // system tables and controller
  if (ncell > 1) b += nc * (4 + 8 + 3 * (4 + 8));            // system CSR (about 3 entries a row)
  if (cell_type == IO && ncell > 1) b += 4LL * ncell * (4 + 4 + 8);  // gap edges
  return b;
}

// ------------------------------------------------- gbrkc_advance_noalloc
// gbrkc_advance without any allocation: the persistent launch's work-queue
// counters and per-CTA timestamps come from the static scratch of
// noalloc.cu, host-side buffers are fixed-size locals, and the stopped-system
// check reads the status words with one strided copy per pool chunk.
namespace {

template <typename R>
int launch_mega_static(gbrkc_engine *E, double t0, int n_iv, int iv0, int init, unsigned long long *scratch) {
  MegaView<R> M{};
  const int end = mega_pools<R>(E, M);
  if (end > NOALLOC_MAX_CTAS)
    return fail(GBRKC_EINVAL, "persistent launch of %d CTAs exceeds the static scratch (%d CTAs)", end,
                NOALLOC_MAX_CTAS);
  if (end > E->mega_grid || end <= 0)
    return fail(GBRKC_ESTATE, "persistent launch: %d role CTAs for a grid of %d", end, E->mega_grid);
  M.gr_nc4 = E->pools[GR].team == TEAM_LANE4;
  M.lane_warps = 0;
  M.lane_extra = 0;
  if (E->role_ctas[GR] > 0) {
    // the role split may have moved since the warps were fitted: at most 8
    // warps a CTA (lanes take further systems in turn)
    E->gr_warps = std::max(1, std::min(E->gr_warps, (MEGA_BLOCK / 32) * E->role_ctas[GR]));
    M.lane_warps = E->gr_warps / E->role_ctas[GR];
    M.lane_extra = E->gr_warps % E->role_ctas[GR];
    if (M.lane_warps + (M.lane_extra > 0) > MEGA_BLOCK / 32)
      return fail(GBRKC_ESTATE, "persistent launch: %d granule warps do not fit %d CTAs", E->gr_warps,
                  E->role_ctas[GR]);
  }
  if (E->role_ctas[GR] > 0 &&
      (!E->pools[GR].ws_in_smem ||
       E->mega_smem < (size_t)MEGA_BLOCK * (size_t)E->pools[GR].ws_tile * sizeof(double)))
    return fail(GBRKC_ESTATE, "persistent launch: granule workspaces do not fit its shared memory");
  M.queue = (int *)scratch;
  M.t_start = scratch + NOALLOC_QUEUE_WORDS;
  M.t_end = scratch + NOALLOC_QUEUE_WORDS + NOALLOC_MAX_CTAS;
  cudaStream_t st = E->streams[0];
  // the counters must start at zero; the stamps are all rewritten
  CUDA_TRY(cudaMemsetAsync(M.queue, 0, NOALLOC_QUEUE_WORDS * sizeof(unsigned long long), st));
  CUDA_TRY(cudaEventRecord(E->ev_start, st));
  int rc = launch_mega<R>(M, end, E->mega_smem, st, t0, n_iv, iv0, init);
  if (rc) return fail(GBRKC_ECUDA, "persistent launch: %s", cudaGetErrorString((cudaError_t)rc));
  CUDA_TRY(cudaEventRecord(E->ev_end, st));
  CUDA_TRY(cudaEventSynchronize(E->ev_end));
  CUDA_TRY(cudaEventElapsedTime(&E->last_ms, E->ev_start, E->ev_end));
  if (init) return 0;
  unsigned long long ts[NOALLOC_MAX_CTAS], te[NOALLOC_MAX_CTAS];
  CUDA_TRY(cudaMemcpy(ts, M.t_start, end * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(te, M.t_end, end * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  unsigned long long t_first = ~0ull;
  for (int b = 0; b < end; b++) t_first = std::min(t_first, ts[b]);
  double role_ms[NTYPES] = {};
  int b = 0;
  for (int t = 0; t < NTYPES; t++) {
    unsigned long long last = t_first;
    for (int k = 0; k < E->role_ctas[t]; k++, b++) last = std::max(last, te[b]);
    role_ms[t] = E->role_ctas[t] ? (double)(last - t_first) * 1e-6 : 0.0;
    E->last_kernel_ms[t] = (float)role_ms[t];
  }
  if (n_iv > 0) rebalance_roles(E, role_ms, true);
  return 0;
}

}  // namespace

extern "C" int gbrkc_advance_noalloc(gbrkc_engine *E, double t0, int n_iv) {
  if (!E || n_iv < 0) return fail(GBRKC_EINVAL, "bad arguments");
  if (!E->built) return fail(GBRKC_ESTATE, "engine not built");
  if (E->sv.n > 0) return fail(GBRKC_EINVAL, "engines with synapses step through gbrkc_advance");
  fit_granule_warps(E);
  const int iv0 = E->soma_iv;
  for (int t = 0; t < NTYPES; t++) {
    PoolHost &P = E->pools[t];
    double *so = (E->soma_cap > 0 && iv0 + n_iv <= E->soma_cap) ? P.d_soma : nullptr;
    P.vd.soma_out = so;
    P.vf.soma_out = so;
  }
  int rc;
  for (int init = E->pending_init ? 1 : 0; init >= 0; init--) {
    // systems reset since the last call are initialised (only they) first
    const int n = init ? 0 : n_iv;
    if (E->mega) {
      unsigned long long *scratch = E->d_static_scratch;
      if (!scratch) return fail(GBRKC_ESTATE, "static scratch address not set up");
      rc = (E->precision == GBRKC_FP64) ? launch_mega_static<double>(E, t0, n, iv0, init, scratch)
                                        : launch_mega_static<float>(E, t0, n, iv0, init, scratch);
    } else {
      // one launch per pool: those kernels use no scratch beyond the engine's state
      rc = launch_all(E, t0, n, iv0, init);
    }
    if (rc) return rc;
    if (init) E->pending_init = false;
  }
  if (E->soma_cap > 0) E->soma_iv += n_iv;
  // stopped systems: their status words and interval budgets (adjacent in
  // Ctl), read in chunks with a strided copy; the granule systems with work
  // left are counted as gbrkc_advance counts them, for the next launch's
  // granule warps
  static_assert(offsetof(Ctl, iv_left) == offsetof(Ctl, status) + sizeof(int), "status and iv_left adjacent");
  int stopped = 0, first_id = -1, first_status = 0;
  constexpr int CHUNK = 512;
  int word[2 * CHUNK];
  for (int t = 0; t < NTYPES; t++) {
    PoolHost &P = E->pools[t];
    const int nsys = (int)P.systems.size();
    long active = 0;
    for (int i0 = 0; i0 < nsys; i0 += CHUNK) {
      const int cnt = std::min(CHUNK, nsys - i0);
      CUDA_TRY(cudaMemcpy2D(word, 2 * sizeof(int), (const char *)(P.d_ctl + i0) + offsetof(Ctl, status),
                            sizeof(Ctl), 2 * sizeof(int), cnt, cudaMemcpyDeviceToHost));
      for (int i = 0; i < cnt; i++) {
        const int status = word[2 * i], iv_left = word[2 * i + 1];
        active += (status == 0 && iv_left != 0);
        if (status) {
          if (!stopped++) { first_id = P.systems[i0 + i]; first_status = status; }
        }
      }
    }
    if (t == GR && nsys > 0) E->gr_active = active;
  }
  if (stopped)
    return fail(GBRKC_ESOLVER, "%d system(s) are stopped (first: system %d, status %d); the others advanced", stopped,
                first_id, first_status);
  return 0;
}

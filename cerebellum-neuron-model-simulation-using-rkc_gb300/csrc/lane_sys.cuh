// Register-resident RKC integrator for single-cell systems of exactly NC
// compartments (the granule cell of the mixed workload has 4): one system per
// thread, the five RKC vectors and the current vector b in registers.
//
// The arithmetic is Sys's (integrator.cuh) operation for operation, so the
// results are bit-identical to it and to the oracle.  What changes is where
// the data lives: the reference rotates its five buffers by index
// (solve_rkc.cu:862-904, 1028-1034); here every logical vector is its own
// register array and a rotation moves values between them.  The system's
// buffer map (Ctl::map) stays as it was loaded and is used only to place the
// vectors back into the workspace at write-back, so readers of the workspace
// see the same logical contents.  On GB300 a lone warp runs this code as a
// serial instruction stream (each dependent FP64 operation ~64 cycles), so
// the instruction count per step attempt is what sets the pace; keeping the
// state in registers removes the address arithmetic and the shared-memory
// traffic of the generic path.
//
// Used for advancing only; initialisation goes through Sys.
#pragma once
#include "integrator.cuh"

namespace gbrkc {

template <int CT, typename R, int NC, int LS>
struct LaneSys {
  const PoolView<R> &P;
  int s, off, cell0;
  // the template's axial operator, dense, in this lane's shared-memory slot
  // (element e at Gs[e * LS]: G(i, j) at e = i * NC + j, 1/Cm(i) at
  // NC * NC + i), and which entries the CSR has (bit i * NC + j of gmask;
  // the CSR holds no duplicates and no diagonal).  Rows are visited in
  // ascending column order, the CSR's order.
  double *Gs;
  unsigned gmask;
  double y[NC], yn[NC], fn[NC], v1[NC], v2[NC], b[NC];
  Ctl c;
  double t0;
  int k_iv, n_iv, iv0, rej_run;
  long long attempts0;

  static_assert(NC * NC + NC <= WS_VECS * ((NC + 1) & ~1), "operator must fit the lane's workspace slot");
  __device__ LaneSys(const PoolView<R> &P_, double *slot) : P(P_), Gs(slot) {}

  // Take system s_ (single cell, template operator, NC compartments) from
  // its workspace and controller record.
  __device__ __forceinline__ void load(int s_) {
    s = s_;
    off = P.sys_off[s];
    cell0 = P.sys_cell0[s];
    const int t = P.sys_tmpl[s];
    const int *row = P.t_row + P.t_row0[t], *col = P.t_col + P.t_nz0[t];
    const double *g = P.t_g + P.t_nz0[t], *invcm = P.t_invcm + P.t_cm0[t];
    gmask = 0u;
#pragma unroll
    for (int i = 0; i < NC; i++) {
      Gs[(NC * NC + i) * LS] = __ldg(invcm + i);
      const int r0 = __ldg(row + i), r1 = __ldg(row + i + 1);
      for (int k = r0; k < r1; k++) {
        const int j = __ldg(col + k);
        Gs[(i * NC + j) * LS] = __ldg(g + k);
        gmask |= 1u << (i * NC + j);
      }
    }
    c = P.ctl[s];
    const double *ws = P.ws + P.sys_ws[s];
    constexpr int NCP = (NC + 1) & ~1;
#pragma unroll
    for (int i = 0; i < NC; i++) {
      y[i] = ws[c.map[LY] * NCP + i];
      yn[i] = ws[c.map[LYN] * NCP + i];
      fn[i] = ws[c.map[LFN] * NCP + i];
      v1[i] = ws[c.map[LV1] * NCP + i];
      v2[i] = ws[c.map[LV2] * NCP + i];
      b[i] = ws[WS_B * NCP + i];
    }
  }

  __device__ __forceinline__ void store() const {
    double *ws = P.ws + P.sys_ws[s];
    constexpr int NCP = (NC + 1) & ~1;
#pragma unroll
    for (int i = 0; i < NC; i++) {
      ws[c.map[LY] * NCP + i] = y[i];
      ws[c.map[LYN] * NCP + i] = yn[i];
      ws[c.map[LFN] * NCP + i] = fn[i];
      ws[c.map[LV1] * NCP + i] = v1[i];
      ws[c.map[LV2] * NCP + i] = v2[i];
      ws[WS_B * NCP + i] = b[i];
    }
    P.ctl[s] = c;
  }

  // dydt at compartment i (Sys::rhs): the CSR's terms in its order; an
  // absent entry is skipped (the operator is the same for every lane of a
  // pool of one template, so the test does not diverge)
  __device__ __forceinline__ double rhs(const double (&u)[NC], int i) const {
    double d = -(b[i]);
    const double ui = u[i];
#pragma unroll
    for (int j = 0; j < NC; j++)
      if (j != i && ((gmask >> (i * NC + j)) & 1u)) d = fma(Gs[(i * NC + j) * LS], u[j] - ui, d);
    return d * Gs[(NC * NC + i) * LS];
  }

  __device__ __forceinline__ static double sumsq(const double (&a)[NC]) {
    double q[NC];
#pragma unroll
    for (int i = 0; i < NC; i++) q[i] = a[i] * a[i];
    return tree_regs<NC>(q);
  }

  // Sys::rkcrho
  __device__ __forceinline__ void rkcrho() {
    const double uround = UROUND, sqrtu = sqrt(UROUND), small = 1.0 / 0.125;
    double *ede = P.ede + off;
    double e[NC];
#pragma unroll
    for (int i = 0; i < NC; i++) e[i] = ede[i];
    double sprad_old[3] = {0.0, 0.0, 0.0};
    c.n_rho++;
    const double ynrm = sqrt(sumsq(yn));
    const double vnrm = sqrt(sumsq(e));
    double dynrm;
    if (ynrm != 0.0 && vnrm != 0.0) {
      dynrm = ynrm * sqrtu;
      const double al = dynrm / vnrm;
#pragma unroll
      for (int i = 0; i < NC; i++) v1[i] = fma(al, e[i], yn[i]);
    } else if (ynrm != 0.0) {
      dynrm = ynrm * sqrtu;
#pragma unroll
      for (int i = 0; i < NC; i++) v1[i] = fma(sqrtu, yn[i], yn[i]);
    } else if (vnrm != 0.0) {
      dynrm = uround;
      const double al = dynrm / vnrm;
#pragma unroll
      for (int i = 0; i < NC; i++) v1[i] = al * e[i];
    } else {
      dynrm = uround;
#pragma unroll
      for (int i = 0; i < NC; i++) v1[i] = dynrm;
    }
    double sigma = 0.0, sigmal;
    for (int iter = 0; iter < RHO_ITMAX; iter++) {
      c.n_rho_iter++;
      double q[NC];
#pragma unroll
      for (int i = 0; i < NC; i++) {
        v2[i] = rhs(v1, i);
        const double dm = -1.0 * fn[i] + v2[i];
        q[i] = dm * dm;
      }
      const double dfnrm = sqrt(tree_regs<NC>(q));
      sigmal = sigma;
      sigma = dfnrm / dynrm;
      sprad_old[0] = sprad_old[1];
      sprad_old[1] = sprad_old[2];
      sprad_old[2] = c.sprad;
      c.sprad = 1.2 * sigma;
      if (iter >= 1 && fabs(sigma - sigmal) <= ((sigma > small) ? sigma : small) * 0.001) {
#pragma unroll
        for (int i = 0; i < NC; i++) ede[i] = -1.0 * yn[i] + v1[i];
        return;
      }
      if (iter > RHO_ITMAX / 2) {
        if ((fabs(sprad_old[2] - sprad_old[0]) < 0.00001) && (fabs(sprad_old[1] - c.sprad) < 0.00001)) {
          c.sprad = (c.sprad + sprad_old[2]) / 2.0;
#pragma unroll
          for (int i = 0; i < NC; i++) ede[i] = -1.0 * yn[i] + v1[i];
          return;
        }
      }
      if (dfnrm != 0.0) {
        const double al = dynrm / dfnrm;
#pragma unroll
        for (int i = 0; i < NC; i++) v1[i] = fma(al, fn[i] - v2[i], yn[i]);
      } else {
        const int idx = iter % NC;
#pragma unroll
        for (int i = 0; i < NC; i++)
          if (i == idx) v1[i] = 2.0 * yn[i] - v1[i];
      }
    }
    c.idid = 6;
  }

  // Sys::step, the buffer rotations as moves
  __device__ __forceinline__ bool step(double h, int m) {
    if (m > P.coef_mmax) {
      c.status |= ST_COEF_TABLE;
      return false;
    }
    const double *T = P.coef + P.coef_off[m];
    {
      const double hm = h * __ldg(T);
#pragma unroll
      for (int i = 0; i < NC; i++) {
        v2[i] = yn[i];
        v1[i] = fma(hm, fn[i], yn[i]);
      }
    }
    for (int j = 1; j < m; j++) {
      const double *q = T + 1 + 5 * (j - 1);
      const double mu = __ldg(q), nu = __ldg(q + 1), omn = __ldg(q + 2), mus = __ldg(q + 3), ajm1 = __ldg(q + 4);
      const double hm = h * mus;
      double out[NC];
#pragma unroll
      for (int i = 0; i < NC; i++) {
        const double f = rhs(v1, i);
        double t = mu * v1[i];
        t = fma(nu, v2[i], t);
        t = fma(omn, yn[i], t);
        const double u = fma(-ajm1, fn[i], f);
        out[i] = fma(hm, u, t);
      }
      // written to y, then (v2, v1, y) <- (v1, y, v2)
#pragma unroll
      for (int i = 0; i < NC; i++) {
        y[i] = v2[i];
        v2[i] = v1[i];
        v1[i] = out[i];
      }
    }
    // (y, v1, v2) <- (v1, v2, y)
#pragma unroll
    for (int i = 0; i < NC; i++) {
      const double t = y[i];
      y[i] = v1[i];
      v1[i] = v2[i];
      v2[i] = t;
    }
    c.n_stage += m;
    return true;
  }

  // Sys::attempt.  In mixed precision (R = float) the controller's scalar
  // chain runs in FP32: the error terms' quotients, their norm and its cube
  // root, the stage count's square root and the step-size ratios.  The step
  // size, the time, the stage recurrence and the accept/reject comparison
  // stay FP64.  A lone granule warp is a latency-bound serial chain, and
  // FP64 square roots, divisions and the cube root's Newton steps are its
  // longest links; in FP32 they change the step sizes by about 1e-7
  // relative, the size of the differences FP32 gating already makes.
  static constexpr bool FAST = !std::is_same<R, double>::value;

  __device__ __forceinline__ int attempt() {
    const double hmax = H_MAX, hmin = c.hmin;
    if (c.newspc) {
      rkcrho();
      c.jacatt = 1;
    }
    c.last = 0;
    if (1.1 * c.absh >= fabs(c.tend - c.lt)) {
      c.absh = fabs(c.tend - c.lt);
      c.last = 1;
    }
    double marg;
    if constexpr (FAST)
      marg = (double)sqrtf((float)(1.54 * c.absh * c.sprad + 1.0));
    else
      marg = sqrt(1.54 * c.absh * c.sprad + 1.0);
    if (!(marg < 1.0e9)) {
      c.status |= ST_NAN;
      return Sys<CT, R, BlockTeam>::ATT_FAIL;
    }
    int m = 1 + (int)(marg);
    if (m > c.mmax) {
      m = (int)c.mmax;
      c.absh = (m * m - 1) / (1.54 * c.sprad);
      c.last = 0;
    }
    double h = 1.0 * c.absh;
    if (h <= hmin) h = hmin;
    if (!step(h, m)) return Sys<CT, R, BlockTeam>::ATT_FAIL;
    c.n_steps++;
    double err, cr;
    if constexpr (FAST) {
      const double h04 = 0.4 * h;
      float q[NC];
#pragma unroll
      for (int i = 0; i < NC; i++) {
        const double f = rhs(y, i);
        v1[i] = f;
        const double ay = fabs(y[i]), ayn = fabs(yn[i]);
        const double wt = fma(c.tol, (ay > ayn) ? ay : ayn, c.tol);
        const double est = fma(h04, fn[i] + f, 0.8 * (yn[i] - y[i]));
        const float qv = (float)est / (float)wt;
        q[i] = qv * qv;
      }
      float e2 = q[0];
#pragma unroll
      for (int i = 1; i < NC; i++) e2 += q[i];
      const float ef = sqrtf(e2 * (1.0f / (float)NC));
      err = (double)ef;
      cr = (double)cbrtf(ef);
    } else {
      const double h04 = 0.4 * h;
      double q[NC];
#pragma unroll
      for (int i = 0; i < NC; i++) {
        const double f = rhs(y, i);
        v1[i] = f;
        const double ay = fabs(y[i]), ayn = fabs(yn[i]);
        const double wt = fma(c.tol, (ay > ayn) ? ay : ayn, c.tol);
        const double est = fma(h04, fn[i] + f, 0.8 * (yn[i] - y[i]));
        const double qv = est / wt;
        q[i] = qv * qv;
      }
      err = tree_regs<NC>(q);
      if ((NC & (NC - 1)) == 0)
        err = sqrt(err * (1.0 / (double)NC));
      else
        err = sqrt(err / (double)NC);
      cr = 0.0;
    }
    if (!(err == err)) {
      c.status |= ST_NAN;
      return Sys<CT, R, BlockTeam>::ATT_FAIL;
    }
    if constexpr (!FAST) cr = cm_cbrt(err);
    if (err > 1.0) {
      if constexpr (FAST)
        c.absh = c.absh * (double)(0.8f / (float)cr);
      else
        c.absh = 0.8 * c.absh / cr;
      c.n_rej++;
      if (c.absh < hmin) {
        c.idid = 4;
      } else {
        c.newspc = !c.jacatt;
        if (++rej_run >= RKCLOW_LOOP_CAP) {
          c.status |= ST_LOOP_CAP;
          return Sys<CT, R, BlockTeam>::ATT_FAIL;
        }
        return Sys<CT, R, BlockTeam>::ATT_REJECT;
      }
    }
    rej_run = 0;
    c.naccpt += 1;
    c.lt += h;
    c.gt = c.lt;
    c.jacatt = 0;
    c.newspc = 0;
    c.hw0 = h;
    c.hw1 = c.lt;
    // (v2, fn, v1, yn, y) <- (fn, v1, yn, y, v2)
#pragma unroll
    for (int i = 0; i < NC; i++) {
      const double t = v2[i];
      v2[i] = fn[i];
      fn[i] = v1[i];
      v1[i] = yn[i];
      yn[i] = y[i];
      y[i] = t;
    }
    if constexpr (FAST) {
      float fac = 10.0f;
      const float crf = (float)cr;
      if (c.naccpt == 1) {
        if (0.8f < fac * crf) fac = 0.8f / crf;
      } else {
        const float temp1 = 0.8f * (float)c.absh * (float)c.cbrt_errold;
        const float temp2 = fabsf((float)c.hold) * (crf * crf);
        if (temp1 < fac * temp2) fac = temp1 / temp2;
      }
      c.absh = (double)((0.1f > fac) ? 0.1f : fac) * c.absh;
    } else {
      double fac = 10.0, temp1, temp2;
      if (c.naccpt == 1) {
        temp2 = cr;
        if (0.8 < fac * temp2) fac = 0.8 / temp2;
      } else {
        temp1 = 0.8 * c.absh * c.cbrt_errold;
        temp2 = fabs(c.hold) * (cr * cr);
        if (temp1 < fac * temp2) fac = temp1 / temp2;
      }
      c.absh = ((0.1 > fac) ? 0.1 : fac) * c.absh;
    }
    c.cbrt_errold = cr;
    {
      const double mn = fmin(hmax, c.absh);
      c.absh = (hmin > mn) ? hmin : mn;
    }
    c.errold = err;
    c.hold = h;
    c.idid = c.last ? 1 : 2;
    return Sys<CT, R, BlockTeam>::ATT_ACCEPT;
  }

  // Sys::ion_and_b for a single cell (no gap junctions)
  __device__ __forceinline__ void ion_due() {
#pragma unroll
    for (int i = 0; i < NC; i++) b[i] = comp_ion_b<CT, R>(P, off + i, y[i], c.sum_dt, true);
    c.n_ion++;
    c.sum_dt = 0.0;
  }

  __device__ __forceinline__ int begin_interval(double t) {
    if (P.stim_on) {
      const int comp = P.stim_comp[cell0];
      if (comp >= 0) {
        const long gi = off + comp;
        P.iext[gi] = 0;
        if (P.stim_t0[cell0] <= t && t < P.stim_t1[cell0]) P.iext[gi] = P.stim_amp[cell0];
      }
    }
    attempts0 = c.n_steps;
    rej_run = 0;
    return (c.sum_dt != 0.0) ? TICK_ION : TICK_MORE;
  }

  __device__ __forceinline__ void end_interval() {
    const double hlast = c.hw0, tlast = c.hw1 - hlast;
    const double sv = (c.gt_old - tlast) / hlast;
    const double a1 = (1.0 + 2.0 * sv) * (sv - 1.0) * (sv - 1.0);
    const double a2 = (3.0 - 2.0 * sv) * sv * sv;
    const double b1 = hlast * sv * (sv - 1.0) * (sv - 1.0);
    const double b2 = hlast * (sv - 1.0) * sv * sv;
#pragma unroll
    for (int i = 0; i < NC; i++) P.vnew[off + i] = fma(b2, fn[i], fma(b1, v2[i], fma(a2, yn[i], a1 * v1[i])));
    c.tend += H_MAX;
    if (P.soma_out)
      for (int k = 0; k < P.rec_w; k++)
        P.soma_out[((long)(iv0 + k_iv) * P.ncell_pool + cell0) * P.rec_w + k] = P.vnew[P.cell_soma[cell0] + k];
    if (P.spk_prev) log_spike(P, cell0, t0 + (k_iv + 1) * H_MAX);
    if (c.iv_left > 0) c.iv_left--;
  }

  __device__ __forceinline__ int start(double t, int n, int iv0_global) {
    if (c.iv_left >= 0 && n > c.iv_left) n = c.iv_left;
    t0 = t;
    n_iv = n;
    iv0 = iv0_global;
    k_iv = 0;
    if (c.status != 0 || n <= 0) return TICK_DONE;
    return begin_interval(t0);
  }

  // Sys::tick
  __device__ __forceinline__ int tick() {
    const int a = attempt();
    if (a == Sys<CT, R, BlockTeam>::ATT_REJECT) return TICK_MORE;
    if (a == Sys<CT, R, BlockTeam>::ATT_FAIL) return TICK_DONE;
    if (c.n_steps - attempts0 > STEPS_PER_INTERVAL_CAP) {
      c.status |= ST_LOOP_CAP;
      return TICK_DONE;
    }
    c.sum_dt += c.gt - c.gt_old;
    c.gt_old = c.gt;
    const bool ge = (CT == GO || CT == PKJ);
    const bool trig = ge ? (c.sum_dt >= c.integ) : (c.sum_dt > c.integ);
    if (c.idid == 2.0) return trig ? TICK_ION : TICK_MORE;
    if (c.idid != 1.0) {
      c.status |= ST_IDID;
      return TICK_DONE;
    }
    end_interval();
    if (++k_iv >= n_iv) return TICK_DONE;
    return begin_interval(t0 + k_iv * H_MAX);
  }
};

// run_lanes (integrator.cuh) with the state in registers for advancing:
// systems from *q or the static sequence first, first + stride, ...; parked
// ion updates run together for the warp.
template <int CT, typename R, int BLOCK, int NC>
__device__ __forceinline__ void run_lanes_regs(const PoolView<R> &P, int *q, int first, int stride, double *smem,
                                               double t0, int n_iv, int iv0_global, bool init) {
  if (init || n_iv <= 0) {
    run_lanes<CT, R, BLOCK, NC>(P, q, first, stride, smem, t0, n_iv, iv0_global, init);
    return;
  }
  LaneSys<CT, R, NC, BLOCK> S(P, smem + threadIdx.x);
  int s = ((int)(threadIdx.x & 31) >= P.lanes) ? P.nsys : (q ? atomicAdd(q, 1) : first);
  int r = TICK_DONE;
  auto acquire = [&]() {
    while (s < P.nsys) {
      if (system_selected(P.ctl[s], false, n_iv)) {
        S.load(s);
        r = S.start(t0, n_iv, iv0_global);
        if (r != TICK_DONE) return;
        S.store();
      }
      s = q ? atomicAdd(q, 1) : s + stride;
    }
    r = TICK_DONE;
  };
  acquire();
  int wait = 0;
  for (;;) {
    __syncwarp();
    const unsigned live = __ballot_sync(0xffffffffu, r != TICK_DONE);
    if (!live) break;
    const unsigned parked = __ballot_sync(0xffffffffu, r == TICK_ION);
    if (parked && (parked == live || ++wait > ION_WAIT_MAX)) {
      wait = 0;
      if (r == TICK_ION) {
        S.ion_due();
        r = TICK_MORE;
      }
      __syncwarp();
    }
    if (r == TICK_MORE) {
      r = S.tick();
      if (r == TICK_DONE) {
        S.store();
        s = q ? atomicAdd(q, 1) : s + stride;
        acquire();
      }
    }
  }
}

}  // namespace gbrkc

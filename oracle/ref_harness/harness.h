/* Interface between the reference-harness pieces (test infrastructure). */
#pragma once
#ifdef __cplusplus
extern "C" {
#endif
struct ref_state {
  int type, n, nc, ncond, nion;
  double *elem[7];  /* v, Ca, Cm, area, connect, compart, i_ext (param.h:20) */
  double *cond[24];
  double *ion[24];
  double *ca2, *rev_ca2, *ca_old, *shell;
};
void ref_init_ion(struct ref_state *s);
void ref_ion_update(struct ref_state *s, double *vnew, double DT);
/* static setup of the reference (initialize_host_* and set_host_*_solve) */
void ref_host_setup(int type, int nx, int ny, struct ref_state *s);
int ref_csr(int type, int nx, int ny, int *row, int *col, double *val, int cap);
#ifdef __cplusplus
}
#endif

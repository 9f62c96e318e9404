// Initial per-compartment state of a cell type (host, libm).
#pragma once
namespace gbrkc {
struct CompInit {
  double v, ca, ca2, rev, ca_old;
  double x[24];
};
void initial_state(int type, double jitter, int comp_type, double g_CaH_io, CompInit *out);
}  // namespace gbrkc

// Per-interval update of the chemical synapses (network mode): the
// reference's mfgr_update, grgo_update, gogr_update and grpkj_update
// (syn.cu:86-111, 263-288, 412-437, 646-668), one thread per synapse, run
// once per 0.125 ms interval after every system has advanced it.
//
// A presynaptic spike is the presynaptic compartment's elem v (the voltage
// its gating last saw) crossing 0 mV upward between two updates; every state
// decays by exp(-RKC_DT / tau) and steps by one on a spike.  Mossy fibres fire
// as Poisson processes, rate * RKC_DT * 1e-3 > U: the reference draws U with
// cuRAND; here U comes from a counter-based generator (the SplitMix64
// finaliser of Steele, Lea & Flood 2014 over seed, synapse and interval), so
// the draws are reproducible and identical in the oracle.
//
// A transmission delay of d intervals (this library's addition; 0 is the
// reference's rule) keeps each synapse's last 64 events in a bit ring: the
// event detected now enters bit 0, and the one detected d intervals ago
// drives the update.
//
// Built with -fmad=false like the other kernel units: the arithmetic is the
// reference's expressions in their order, bit-identical to the oracle.
#include <cuda_runtime.h>

#include "engine.h"
#include "splitmix.h"

namespace gbrkc {

// syn.cuh:11-45
constexpr double G_MFGR_AMPA = 0.18e-9, G_MFGR_NMDA = 0.025e-9;
constexpr double G_GRGO_AMPA = 45.5e-9, G_GRGO_NMDA = 30.0e-9;
constexpr double G_GOGR_GABA = 0.028e-9;
constexpr double G_GRPKJ_AMPA = 0.7e-9;
constexpr double RKC_DT_MS = 0.125;

__device__ __forceinline__ double syn_uniform(unsigned long long seed, long long id, long long interval) {
  return splitmix_uniform(seed, id, interval);
}

__device__ __forceinline__ int delayed(const SynView &S, int id, int f_now) {
  if (!S.ring) return f_now;
  const unsigned long long r = (S.ring[id] << 1) | (unsigned long long)f_now;
  S.ring[id] = r;
  return (int)((r >> S.delay[id]) & 1ull);
}

__global__ void k_syn_update(const __grid_constant__ SynView S, double t, long long interval) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= S.n) return;
  const int kind = S.kind[id];
  if (kind == SYN_MFGR) {
    const int g = S.grp[id];
    const double *r = S.grp_rate + 4 * g;
    const double fr = (r[2] <= t && t < r[3]) ? r[1] : r[0];
    const double u = syn_uniform(S.grp_seed[g], id, interval);
    const int f = delayed(S, id, (fr * RKC_DT_MS * 0.001 > u) ? 1 : 0);
    const double ampa = S.s0[id] * S.decay[0] + f;
    // the NMDA state steps from the already-updated AMPA value (syn.cu:104)
    const double nmda = ampa * S.decay[1] + f;
    S.s0[id] = ampa;
    S.s1[id] = nmda;
    S.val[id] = S.w[id] * (G_MFGR_AMPA * ampa + G_MFGR_NMDA * nmda);
    return;
  }
  const double pv = S.pre_v[S.pre_type[id]][S.pre_gi[id]];
  const int f = delayed(S, id, (pv > 0.0 && S.old_v[id] < 0.0) ? 1 : 0);
  if (kind == SYN_GRGO) {
    const double a = S.s0[id] * S.decay[2] + f;
    const double n1 = S.s1[id] * S.decay[3] + f;
    const double n2 = S.s2[id] * S.decay[4] + f;
    S.s0[id] = a;
    S.s1[id] = n1;
    S.s2[id] = n2;
    S.val[id] = S.w[id] * (G_GRGO_AMPA * a + G_GRGO_NMDA * (0.33 * n1 + 0.67 * n2));
  } else if (kind == SYN_GOGR) {
    const double ga = S.s0[id] * S.decay[5] + f;
    const double gb = S.s1[id] * S.decay[6] + f;
    S.s0[id] = ga;
    S.s1[id] = gb;
    S.val[id] = S.w[id] * G_GOGR_GABA * (0.43 * ga + 0.57 * gb);
  } else {  // SYN_GRPKJ
    const double a = S.s0[id] * S.decay[7] + f;
    S.s0[id] = a;
    S.val[id] = a * S.w[id] * G_GRPKJ_AMPA;
  }
  S.old_v[id] = pv;
}

int launch_syn_update(const SynView &S, void *stream, double t, long long interval) {
  if (S.n <= 0) return 0;
  SynView c = S;
  k_syn_update<<<(S.n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(c, t, interval);
  return (int)cudaGetLastError();
}

}  // namespace gbrkc

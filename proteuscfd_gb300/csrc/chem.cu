// Finite-rate chemistry: mass production rates per node (the per-node
// chemistry of the reacting equation set), one thread per node, the
// mechanism staged in shared memory per block.
//   ChemModel<T>::GetMassProductionRates      ucs/chem.tcc:575
//   Reaction<T>::GetForwardReactionRate       ucs/reaction.tcc:608
//   Reaction<T>::GetEquilibriumReactionRate   ucs/reaction.tcc:629
//   Reaction<T>::GetBackwardReactionRate      ucs/reaction.tcc:683
//   Reaction<T>::GetMassProductionRate        ucs/reaction.tcc:763
//   Species<T>::GetThermoCoeff                ucs/species.tcc:96
// The reference evaluates each reaction's rates once per species it
// produces; here each reaction is evaluated once per node and its
// contribution added to every species it changes, in reaction order, which
// is the order each species' sum has in the reference.
#include "../../include/pcfd.h"

#include <cuda_runtime.h>

#include <cstring>
#include <string>

void pcfd_set_last_error(const std::string& msg);

namespace {

constexpr double kUnivR = 8.31447215;  // ucs/chem_constants.h:5
constexpr double kPref = 101325.0;     // ucs/reaction.tcc:665

struct ChemHandle {
  pcfd_chem_model host;
  pcfd_chem_model* dev = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double *d_rho = nullptr, *d_T = nullptr, *d_w = nullptr;
  long long cap = 0;
};

int cuda_fail(cudaError_t e, const char* what) {
  pcfd_set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? PCFD_ERR_NOMEM : PCFD_ERR_CUDA;
}
#define CHEM_TRY(x, what)                   \
  do {                                      \
    cudaError_t e_ = (x);                   \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

__device__ __forceinline__ bool whole(double v) { return v == floor(v); }

// x^a: small whole exponents (the stoichiometric coefficients of the
// mechanisms, 0..3) by multiplication, which FP64 pow would spend ~20
// operations on; anything else through pow
__device__ __forceinline__ double stoich_pow(double x, double a) {
  if (a == 0.0) return 1.0;
  if (a == 1.0) return x;
  if (a == 2.0) return x * x;
  if (a == 3.0) return x * x * x;
  return pow(x, whole(a) ? (double)(int)a : a);
}

__device__ __forceinline__ const double* thermo_coeff(const pcfd_chem_model& m, int s, double T) {
  if (T < 200.0) return m.nasa_lo[s];
  if (T > 6000.0) return m.nasa_hi[s];
  return T > 1000.0 ? m.nasa_hi[s] : m.nasa_lo[s];
}

__device__ double forward_rate(const pcfd_chem_reaction& r, double T) {
  switch (r.type) {
    case 0: return r.A * exp(-r.EA / (kUnivR * T));
    case 1: return r.A * pow(T, r.n) * exp(-r.EA / (kUnivR * T));
    case 2: return r.A * pow(T, r.n) * exp(-r.EA / T);
    case 3: return r.A * pow(T, r.n);
  }
  return -999.0;
}

__device__ double equilibrium_const(const pcfd_chem_model& m, const pcfd_chem_reaction& r, double T, double logT) {
  double nu = 0.0, d0 = 0.0, d1 = 0.0, d2 = 0.0, d3 = 0.0, d4 = 0.0, d5 = 0.0, d6 = 0.0;
  for (int i = 0; i < r.nlocal; i++) {
    const double* a = thermo_coeff(m, r.global[i], T);
    const double dnu = r.nupp[i] - r.nup[i];
    nu += dnu;
    d0 += dnu * a[0];
    d1 += dnu * a[1];
    d2 += dnu * a[2];
    d3 += dnu * a[3];
    d4 += dnu * a[4];
    d5 += dnu * a[5];
    d6 += dnu * a[6];
  }
  double Kp = exp(d0 * (logT - 1.0) + T * (d1 / 2.0 + T * (d2 / 6.0 + T * (d3 / 12.0 + d4 / 20.0 * T))) - d5 / T + d6);
  double Kc = Kp;
  if (!(fabs(nu) < 1.0e-15)) Kc *= pow(kPref / (kUnivR * T), whole(nu) ? (double)(int)nu : nu);
  return Kc;
}

__global__ void __launch_bounds__(128) k_chem_rates(long long n, const pcfd_chem_model* __restrict__ gm,
                                                    const double* __restrict__ rhoi, const double* __restrict__ Tn,
                                                    double* __restrict__ wdot) {
  __shared__ pcfd_chem_model m;
  {
    // stage the mechanism (about 17 KB) with 8-byte copies
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(gm);
    unsigned long long* dst = reinterpret_cast<unsigned long long*>(&m);
    for (int k = threadIdx.x; k < (int)(sizeof(pcfd_chem_model) / 8); k += blockDim.x) dst[k] = src[k];
  }
  __syncthreads();
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int ns = m.nspecies;
  double X[PCFD_CHEM_MAX_SPECIES], w[PCFD_CHEM_MAX_SPECIES];
  for (int k = 0; k < ns; k++) {
    X[k] = rhoi[p * ns + k] / m.mw[k];
    w[k] = 0.0;
  }
  const double T = Tn[p];
  const double logT = log(T);
  double Xsum = 0.0;
  for (int k = 0; k < ns; k++) Xsum += X[k];
  for (int j = 0; j < m.nreactions; j++) {
    const pcfd_chem_reaction& r = m.rx[j];
    const double Kf = forward_rate(r, T);
    const double Kb = Kf / equilibrium_const(m, r, T, logT);
    double form = 1.0, dest = 1.0;
    for (int l = 0; l < r.nlocal; l++) {
      const double x = X[r.global[l]];
      const double a = r.nup[l], b = r.nupp[l];
      form *= stoich_pow(x, a);
      dest *= stoich_pow(x, b);
    }
    double Mc = 1.0;
    if (r.third_bodies) {
      Mc = Xsum;
      for (int l = 0; l < r.nlocal; l++) Mc += (r.tbeff[l] - 1.0) * X[r.global[l]];
    }
    const double net = Kf * form - Kb * dest;
    for (int l = 0; l < r.nlocal; l++) {
      const double nu = r.nupp[l] - r.nup[l];
      if (nu == 0.0) continue;
      const int g = r.global[l];
      double t = nu * Mc * net;
      t *= m.mw[g];
      w[g] += t;
    }
  }
  for (int k = 0; k < ns; k++) wdot[p * ns + k] = w[k];
}

int validate(const pcfd_chem_model* m) {
  if (m->nspecies < 1 || m->nspecies > PCFD_CHEM_MAX_SPECIES || m->nreactions < 0 ||
      m->nreactions > PCFD_CHEM_MAX_REACTIONS)
    return 0;
  for (int k = 0; k < m->nspecies; k++)
    if (!(m->mw[k] > 0.0)) return 0;
  for (int j = 0; j < m->nreactions; j++) {
    const pcfd_chem_reaction& r = m->rx[j];
    if (r.type < 0 || r.type > 3 || r.nlocal < 0 || r.nlocal > PCFD_CHEM_MAX_LOCAL) return 0;
    for (int l = 0; l < r.nlocal; l++) {
      if (r.global[l] < 0 || r.global[l] >= m->nspecies) return 0;
      for (int q = 0; q < l; q++)
        if (r.global[q] == r.global[l]) return 0;  // one entry per species, as the reference merges them
    }
  }
  return 1;
}

int ensure_io(ChemHandle* c, long long n) {
  if (c->cap >= n) return PCFD_OK;
  cudaFree(c->d_rho);
  cudaFree(c->d_T);
  cudaFree(c->d_w);
  c->d_rho = c->d_T = c->d_w = nullptr;
  c->cap = 0;
  const size_t ns = c->host.nspecies;
  CHEM_TRY(cudaMalloc(&c->d_rho, (size_t)n * ns * sizeof(double)), "chem buffers");
  CHEM_TRY(cudaMalloc(&c->d_T, (size_t)n * sizeof(double)), "chem buffers");
  CHEM_TRY(cudaMalloc(&c->d_w, (size_t)n * ns * sizeof(double)), "chem buffers");
  c->cap = n;
  return PCFD_OK;
}

}  // namespace

extern "C" {

PCFD_API int pcfd_chem_create(const pcfd_chem_model* model, pcfd_chem_t* out) {
  if (!model || !out) {
    pcfd_set_last_error("pcfd_chem_create: null pointer");
    return PCFD_ERR_ARG;
  }
  *out = nullptr;
  if (!validate(model)) {
    pcfd_set_last_error("pcfd_chem_create: model out of range (species, reactions or indices)");
    return PCFD_ERR_ARG;
  }
  ChemHandle* c = new ChemHandle();
  std::memcpy(&c->host, model, sizeof(pcfd_chem_model));
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
  if (e == cudaSuccess) e = cudaMalloc(&c->dev, sizeof(pcfd_chem_model));
  if (e == cudaSuccess) e = cudaMemcpy(c->dev, model, sizeof(pcfd_chem_model), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    int rc = cuda_fail(e, "pcfd_chem_create");
    pcfd_chem_destroy((pcfd_chem_t)c);
    return rc;
  }
  *out = (pcfd_chem_t)c;
  return PCFD_OK;
}

PCFD_API int pcfd_chem_destroy(pcfd_chem_t h) {
  ChemHandle* c = (ChemHandle*)h;
  if (!c) return PCFD_OK;
  if (c->stream) cudaStreamSynchronize(c->stream);
  cudaFree(c->dev);
  cudaFree(c->d_rho);
  cudaFree(c->d_T);
  cudaFree(c->d_w);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return PCFD_OK;
}

PCFD_API int pcfd_chem_production_rates_dev(pcfd_chem_t h, long long n, const double* rhoi, const double* T,
                                            double* wdot, double* ms_out) {
  ChemHandle* c = (ChemHandle*)h;
  if (!c || n < 0 || (n > 0 && (!rhoi || !T || !wdot))) {
    pcfd_set_last_error("pcfd_chem_production_rates_dev: bad arguments");
    return PCFD_ERR_ARG;
  }
  if (n == 0) {
    if (ms_out) *ms_out = 0.0;
    return PCFD_OK;
  }
  CHEM_TRY(cudaEventRecord(c->ev0, c->stream), "chem event");
  k_chem_rates<<<(unsigned)((n + 127) / 128), 128, 0, c->stream>>>(n, c->dev, rhoi, T, wdot);
  CHEM_TRY(cudaGetLastError(), "k_chem_rates launch");
  CHEM_TRY(cudaEventRecord(c->ev1, c->stream), "chem event");
  CHEM_TRY(cudaEventSynchronize(c->ev1), "k_chem_rates");
  if (ms_out) {
    float ms = 0.f;
    CHEM_TRY(cudaEventElapsedTime(&ms, c->ev0, c->ev1), "chem event");
    *ms_out = ms;
  }
  return PCFD_OK;
}

PCFD_API int pcfd_chem_production_rates(pcfd_chem_t h, long long n, const double* rhoi, const double* T,
                                        double* wdot) {
  ChemHandle* c = (ChemHandle*)h;
  if (!c || n < 0 || (n > 0 && (!rhoi || !T || !wdot))) {
    pcfd_set_last_error("pcfd_chem_production_rates: bad arguments");
    return PCFD_ERR_ARG;
  }
  if (n == 0) return PCFD_OK;
  int rc = ensure_io(c, n);
  if (rc) return rc;
  const size_t ns = c->host.nspecies;
  CHEM_TRY(cudaMemcpyAsync(c->d_rho, rhoi, (size_t)n * ns * sizeof(double), cudaMemcpyHostToDevice, c->stream),
           "chem copy");
  CHEM_TRY(cudaMemcpyAsync(c->d_T, T, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->stream), "chem copy");
  rc = pcfd_chem_production_rates_dev(h, n, c->d_rho, c->d_T, c->d_w, nullptr);
  if (rc) return rc;
  CHEM_TRY(cudaMemcpyAsync(wdot, c->d_w, (size_t)n * ns * sizeof(double), cudaMemcpyDeviceToHost, c->stream),
           "chem copy");
  CHEM_TRY(cudaStreamSynchronize(c->stream), "chem sync");
  return PCFD_OK;
}

}  // extern "C"

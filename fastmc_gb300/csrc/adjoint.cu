// adjoint.cu -- guest-framework interaction energy of a guest snapshot and
// its adjoint: dE/d(guest site coordinates) and dE/d(epsilon, sigma, charge
// scale) of every framework atom type.  No counterpart in the reference.
//
// E = sum over guest sites i and framework atoms j within the cutoff of
//       q_i lambda_t q_j r4pie0/epsq erfc(alpha r)/r
//     + 4 eps_it [(sigma_it/r)^12 - (sigma_it/r)^6]
//   + krecip * sum_k a_k 2 Re(S_g(k) conj(S_fw(k))),
// the cross terms of the Ewald sum between the guests and the framework
// (the same k-vectors, a_k and krecip as the trial-move path), in kcal/mol.
// Framework type t carries (eps_t, sigma_t, lambda_t), eps in the FIELD's
// energy unit; guest site type a carries (eps_a, sigma_a) from the FIELD's
// a-a pair; pairs mix by
// Lorentz-Berthelot (eps_it = sqrt(eps_a eps_t), sigma_it = (sigma_a +
// sigma_t)/2); S_fw = sum_t lambda_t S_t with S_t the structure factor of
// the type-t atoms at their FIELD charges.  Orthorhombic cells; FP64.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/fastmc_gb300.h"
#include "device_core.cuh"
#include "fmc_internal.h"

namespace {

using fmc::Error;
using fmc::raise;
using fmcdev::kPi;
using fmcdev::kSqrPi;

#define FMC_ACUDA(x)                                                                \
  do {                                                                              \
    cudaError_t e_ = (x);                                                           \
    if (e_ != cudaSuccess)                                                          \
      ::fmc::raise(FMC_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_));  \
  } while (0)

template <class F>
int aguard(F &&f) {
  try {
    fmc::set_error("");
    return f();
  } catch (const Error &e) {
    fmc::set_error(e.msg);
    return e.code;
  } catch (const std::exception &e) {
    fmc::set_error(e.what());
    return FMC_ERR_INPUT;
  }
}

template <class T>
struct ABuf {
  T *p = nullptr;
  size_t n = 0;
  ABuf() = default;
  ABuf(const ABuf &) = delete;
  ABuf &operator=(const ABuf &) = delete;
  ~ABuf() {
    if (p) cudaFree(p);
  }
  void upload(const std::vector<T> &v) {
    if (p) cudaFree(p);
    p = nullptr;
    n = v.size();
    if (n) {
      FMC_ACUDA(cudaMalloc(&p, n * sizeof(T)));
      FMC_ACUDA(cudaMemcpy(p, v.data(), n * sizeof(T), cudaMemcpyHostToDevice));
    }
  }
  void alloc(size_t count) {
    if (p) cudaFree(p);
    p = nullptr;
    n = count;
    if (n) FMC_ACUDA(cudaMalloc(&p, n * sizeof(T)));
  }
};

constexpr int kAT = 256;       // threads per block
constexpr int kMaxAType = 16;  // framework atom types
constexpr int kMaxASite = 8;   // guest sites

struct AdjConst {
  double L[3], rL[3];
  double alpha, rc2, r4e, rengunit, krecip;
  int nfw, ns, ntype, nk;
  double qs[kMaxASite], eps_s[kMaxASite], sig_s[kMaxASite];
  double par[kMaxAType][3];  // eps_t, sigma_t, lambda_t
};

// Block sum of n doubles per thread into out[0..n) with atomics.
template <int N>
__device__ void block_atomic_sum(double (&v)[N], double *out, double *sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = 0; i < N; ++i) {
    double x = v[i];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[w * N + i] = x;
  }
  __syncthreads();
  if (threadIdx.x < N) {
    double t = 0.0;
    for (int k = 0; k < kAT / 32; ++k) t += sh[k * N + threadIdx.x];
    if (t != 0.0) atomicAdd(out + threadIdx.x, t);
  }
  __syncthreads();
}

// Real-space pairs: blockIdx.y = guest site, threads over framework atoms.
// acc[0] = energy, acc[1 + 3 t + (0, 1, 2)] = dE/d(eps_t, sigma_t, lambda_t).
__global__ void __launch_bounds__(kAT) adj_real_kernel(AdjConst c, const double4 *__restrict__ fw,
                                                       const int *__restrict__ fwt,
                                                       const double *__restrict__ xyz, double *gxyz,
                                                       double *acc) {
  __shared__ double sh[(kAT / 32) * (1 + 3 * kMaxAType)];
  const int i = blockIdx.y, s = i % c.ns;
  const double xi = xyz[3 * i], yi = xyz[3 * i + 1], zi = xyz[3 * i + 2];
  const double qi = c.qs[s], ea = c.eps_s[s], sa = c.sig_s[s];
  double gx = 0.0, gy = 0.0, gz = 0.0;
  double v[1 + 3 * kMaxAType];
  for (int k = 0; k < 1 + 3 * kMaxAType; ++k) v[k] = 0.0;
  for (int j = blockIdx.x * kAT + threadIdx.x; j < c.nfw; j += gridDim.x * kAT) {
    const double4 a = fw[j];
    double dx = xi - a.x, dy = yi - a.y, dz = zi - a.z;
    dx -= c.L[0] * rint(dx * c.rL[0]);
    dy -= c.L[1] * rint(dy * c.rL[1]);
    dz -= c.L[2] * rint(dz * c.rL[2]);
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (r2 >= c.rc2) continue;
    const int t = fwt[j];
    const double r = sqrt(r2), rr = 1.0 / r;
    const double lam = c.par[t][2];
    // Coulomb with the Ewald real-space screening
    const double cq = qi * a.w * c.r4e;
    const double ef = erfc(c.alpha * r) * rr;
    const double dcdr0 = -ef * rr - (2.0 * c.alpha / kSqrPi) * exp(-c.alpha * c.alpha * r2) * rr;
    const double ec0 = cq * ef;  // at lambda_t = 1
    // Lennard-Jones, Lorentz-Berthelot mixing
    const double et = c.par[t][0], st = c.par[t][1];
    // eps in the FIELD's energy unit, the sums in the reference's internal one
    const double eps = sqrt(ea * et) / c.rengunit, sig = 0.5 * (sa + st);
    const double sr2 = sig * sig * rr * rr, sr6 = sr2 * sr2 * sr2;
    const double elj = 4.0 * eps * sr6 * (sr6 - 1.0);
    const double dljdr = 4.0 * eps * (6.0 * sr6 - 12.0 * sr6 * sr6) * rr;
    const double dedr = lam * cq * dcdr0 + dljdr;
    gx += dedr * dx * rr;
    gy += dedr * dy * rr;
    gz += dedr * dz * rr;
    v[0] += lam * ec0 + elj;
    v[1 + 3 * t] += et > 0.0 ? elj / (2.0 * et) : 0.0;
    v[1 + 3 * t + 1] += 0.5 * (24.0 * eps / sig) * (2.0 * sr6 * sr6 - sr6);
    v[1 + 3 * t + 2] += ec0;
  }
  for (int k = 0; k < 1 + 3 * kMaxAType; ++k) v[k] *= c.rengunit;
  double g3[3] = {gx * c.rengunit, gy * c.rengunit, gz * c.rengunit};
  block_atomic_sum(g3, gxyz + 3 * i, sh);
  block_atomic_sum(v, acc, sh);
}

// Per-type framework structure factor at unit charge scale: thread per k.
__global__ void adj_skt_kernel(AdjConst c, const double4 *__restrict__ fw, const int *__restrict__ fwt,
                               const int4 *__restrict__ klmn, double2 *skt) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= c.nk) return;
  const int4 l = klmn[k];
  const double kx = 2.0 * kPi * l.x * c.rL[0], ky = 2.0 * kPi * l.y * c.rL[1],
               kz = 2.0 * kPi * l.z * c.rL[2];
  double re[kMaxAType], im[kMaxAType];
  for (int t = 0; t < c.ntype; ++t) re[t] = im[t] = 0.0;
  for (int j = 0; j < c.nfw; ++j) {
    const double4 a = fw[j];
    double sn, cs;
    sincos(kx * a.x + ky * a.y + kz * a.z, &sn, &cs);
    const int t = fwt[j];
    re[t] += a.w * cs;
    im[t] += a.w * sn;
  }
  for (int t = 0; t < c.ntype; ++t) skt[(size_t)t * c.nk + k] = make_double2(re[t], im[t]);
}

// Guest structure factor and the reciprocal energy / charge-scale
// gradients: thread per k.
__global__ void __launch_bounds__(kAT) adj_recip_k_kernel(AdjConst c, const int4 *__restrict__ klmn,
                                                          const double *__restrict__ akk,
                                                          const double2 *__restrict__ skt,
                                                          const double *__restrict__ xyz, int nsite,
                                                          double2 *sfw, double *acc) {
  __shared__ double sh[(kAT / 32) * (1 + 3 * kMaxAType)];
  const int k = blockIdx.x * kAT + threadIdx.x;
  double v[1 + 3 * kMaxAType];  // the layout of acc
  for (int q = 0; q < 1 + 3 * kMaxAType; ++q) v[q] = 0.0;
  if (k < c.nk) {
    const int4 l = klmn[k];
    const double kx = 2.0 * kPi * l.x * c.rL[0], ky = 2.0 * kPi * l.y * c.rL[1],
                 kz = 2.0 * kPi * l.z * c.rL[2];
    double gr = 0.0, gi = 0.0;
    for (int i = 0; i < nsite; ++i) {
      double sn, cs;
      sincos(kx * xyz[3 * i] + ky * xyz[3 * i + 1] + kz * xyz[3 * i + 2], &sn, &cs);
      const double q = c.qs[i % c.ns];
      gr += q * cs;
      gi += q * sn;
    }
    double fr = 0.0, fi = 0.0;
    const double f = 2.0 * c.krecip * akk[k] * c.rengunit;
    for (int t = 0; t < c.ntype; ++t) {
      const double2 st = skt[(size_t)t * c.nk + k];
      const double lam = c.par[t][2];
      fr += lam * st.x;
      fi += lam * st.y;
      v[1 + 3 * t + 2] = f * (gr * st.x + gi * st.y);  // dE/dlambda_t
    }
    v[0] = f * (gr * fr + gi * fi);
    sfw[k] = make_double2(fr, fi);
  }
  block_atomic_sum(v, acc, sh);
}

// Reciprocal gradient of guest site i: thread per site, loop over k.
__global__ void adj_recip_site_kernel(AdjConst c, const int4 *__restrict__ klmn,
                                      const double *__restrict__ akk, const double2 *__restrict__ sfw,
                                      const double *__restrict__ xyz, int nsite, double *gxyz) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nsite) return;
  const double x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
  const double q = c.qs[i % c.ns];
  double gx = 0.0, gy = 0.0, gz = 0.0;
  for (int k = 0; k < c.nk; ++k) {
    const int4 l = klmn[k];
    const double kx = 2.0 * kPi * l.x * c.rL[0], ky = 2.0 * kPi * l.y * c.rL[1],
                 kz = 2.0 * kPi * l.z * c.rL[2];
    double sn, cs;
    sincos(kx * x + ky * y + kz * z, &sn, &cs);
    const double2 f = sfw[k];
    // d/dr of 2 Re(q e^{ik.r} conj(S_fw)) = -2 q k Im(e^{ik.r} conj(S_fw))
    const double imv = sn * f.x - cs * f.y;
    const double w = -2.0 * c.krecip * akk[k] * q * imv;
    gx += w * kx;
    gy += w * ky;
    gz += w * kz;
  }
  gxyz[3 * i] += gx * c.rengunit;
  gxyz[3 * i + 1] += gy * c.rengunit;
  gxyz[3 * i + 2] += gz * c.rengunit;
}

}  // namespace

struct fmc_adjoint {
  AdjConst c{};
  ABuf<double4> fw;
  ABuf<int> fwt;
  ABuf<int4> klmn;
  ABuf<double> akk;
  ABuf<double2> skt, sfw;
  ABuf<double> acc;
  std::vector<int> type_of_field;  // framework type index -> FIELD unique type
};

extern "C" {

int fmc_adjoint_create(const fmc_system *sys, fmc_adjoint **out) {
  return aguard([&] {
    if (!sys || !out) raise(FMC_ERR_ARG, "null argument");
    const fmc::System &s = sys->s;
    if (s.imcon != 1 && s.imcon != 2) raise(FMC_ERR_INPUT, "the adjoint supports orthorhombic cells");
    if (s.ntpguest != 1) raise(FMC_ERR_INPUT, "the adjoint takes one guest type");
    auto a = new fmc_adjoint();
    std::unique_ptr<fmc_adjoint> hold(a);
    AdjConst &c = a->c;
    for (int d = 0; d < 3; ++d) {
      c.L[d] = s.cell[4 * d];
      c.rL[d] = 1.0 / c.L[d];
    }
    c.alpha = s.alpha;
    c.rc2 = s.rcut * s.rcut;
    c.r4e = fmc::kR4pie0 / s.epsq;
    c.rengunit = 1.0 / s.engunit;
    c.krecip = 2.0 * (2.0 * fmc::kPi / s.volm) * fmc::kR4pie0 / s.epsq;
    // LJ 12-6 parameters of a type from its self pair
    auto self_lj = [&](int t, double &eps, double &sig) {
      const int iv = s.lstvdw[fmc::loc2(t, t)];
      if (iv < 1 || iv > s.ntpvdw || s.ltpvdw[iv] != 2)
        raise(FMC_ERR_INPUT, "the adjoint needs a 12-6 LJ self pair for every atom type");
      eps = s.prmvdw[iv][1] / s.engunit;  // back to the FIELD's unit
      sig = s.prmvdw[iv][2];
    };
    const fmc::MolType &fwm = s.mol[s.fw_mol];
    std::vector<int> idx(s.ntpatm + 2, -1);
    for (int i = 0; i < fwm.natoms; ++i) {
      const int t = fwm.ltp[i];
      if (idx[t] < 0) {
        if ((int)a->type_of_field.size() >= kMaxAType) raise(FMC_ERR_CAPACITY, "too many framework types");
        idx[t] = (int)a->type_of_field.size();
        a->type_of_field.push_back(t);
      }
    }
    c.ntype = (int)a->type_of_field.size();
    for (int k = 0; k < c.ntype; ++k) {
      self_lj(a->type_of_field[k], c.par[k][0], c.par[k][1]);
      c.par[k][2] = 1.0;
    }
    const fmc::MolType &gm = s.mol[s.locguest[1]];
    if (gm.natoms > kMaxASite) raise(FMC_ERR_CAPACITY, "guest has too many sites");
    c.ns = gm.natoms;
    for (int i = 0; i < gm.natoms; ++i) {
      c.qs[i] = gm.chg[i];
      self_lj(gm.ltp[i], c.eps_s[i], c.sig_s[i]);
    }
    std::vector<double4> fw;
    std::vector<int> fwt;
    for (int m = 0; m < fwm.nummols; ++m)
      for (int i = 0; i < fwm.natoms; ++i) {
        const double *p = &fwm.xyz[3 * ((size_t)m * fwm.natoms + i)];
        fw.push_back(make_double4(p[0], p[1], p[2], fwm.chg[i]));
        fwt.push_back(idx[fwm.ltp[i]]);
      }
    c.nfw = (int)fw.size();
    a->fw.upload(fw);
    a->fwt.upload(fwt);
    std::vector<int4> kl(s.newld);
    for (int k = 0; k < s.newld; ++k) kl[k] = make_int4(s.kl[k], s.km[k], s.kn[k], 0);
    c.nk = s.newld;
    a->klmn.upload(kl);
    a->akk.upload(s.akk);
    a->skt.alloc((size_t)c.ntype * std::max(1, c.nk));
    a->sfw.alloc(std::max(1, c.nk));
    a->acc.alloc(1 + 3 * kMaxAType);
    if (c.nk) {
      adj_skt_kernel<<<(c.nk + 127) / 128, 128>>>(c, a->fw.p, a->fwt.p, a->klmn.p, a->skt.p);
      FMC_ACUDA(cudaGetLastError());
      FMC_ACUDA(cudaDeviceSynchronize());
    }
    *out = hold.release();
    return FMC_OK;
  });
}

int fmc_adjoint_info(const fmc_adjoint *a, int *ntype, int *nsite, double *base) {
  return aguard([&] {
    if (!a) raise(FMC_ERR_ARG, "null argument");
    if (ntype) *ntype = a->c.ntype;
    if (nsite) *nsite = a->c.ns;
    if (base)
      for (int t = 0; t < a->c.ntype; ++t)
        for (int q = 0; q < 3; ++q) base[3 * t + q] = a->c.par[t][q];
    return FMC_OK;
  });
}

int fmc_adjoint_eval(fmc_adjoint *a, int nmol, const double *xyz, const double *params,
                     double *energy, double *gxyz, double *gparams) {
  return aguard([&] {
    if (!a || !xyz || !params || !energy || !gxyz || !gparams) raise(FMC_ERR_ARG, "null argument");
    if (nmol < 0) raise(FMC_ERR_ARG, "negative molecule count");
    AdjConst c = a->c;
    for (int t = 0; t < c.ntype; ++t)
      for (int q = 0; q < 3; ++q) c.par[t][q] = params[3 * t + q];
    for (int t = 0; t < c.ntype; ++t)
      if (!(c.par[t][0] >= 0.0) || !(c.par[t][1] > 0.0)) raise(FMC_ERR_ARG, "epsilon >= 0 and sigma > 0 required");
    const int nsite = nmol * c.ns;
    if (nsite > 65535) raise(FMC_ERR_CAPACITY, "at most 65535 guest sites");
    FMC_ACUDA(cudaMemset(a->acc.p, 0, a->acc.n * sizeof(double)));
    FMC_ACUDA(cudaMemset(gxyz, 0, (size_t)nsite * 3 * sizeof(double)));
    if (nsite > 0) {
      dim3 grid((c.nfw + kAT - 1) / kAT, nsite);
      if (grid.x > 64) grid.x = 64;
      adj_real_kernel<<<grid, kAT>>>(c, a->fw.p, a->fwt.p, xyz, gxyz, a->acc.p);
      FMC_ACUDA(cudaGetLastError());
      if (c.nk) {
        adj_recip_k_kernel<<<(c.nk + kAT - 1) / kAT, kAT>>>(c, a->klmn.p, a->akk.p, a->skt.p, xyz, nsite,
                                                           a->sfw.p, a->acc.p);
        FMC_ACUDA(cudaGetLastError());
        adj_recip_site_kernel<<<(nsite + 127) / 128, 128>>>(c, a->klmn.p, a->akk.p, a->sfw.p, xyz, nsite,
                                                             gxyz);
        FMC_ACUDA(cudaGetLastError());
      }
    }
    std::vector<double> acc(a->acc.n);
    FMC_ACUDA(cudaMemcpy(acc.data(), a->acc.p, acc.size() * sizeof(double), cudaMemcpyDeviceToHost));
    *energy = acc[0];
    for (int t = 0; t < c.ntype; ++t)
      for (int q = 0; q < 3; ++q) gparams[3 * t + q] = acc[1 + 3 * t + q];
    return FMC_OK;
  });
}

int fmc_adjoint_destroy(fmc_adjoint *a) {
  delete a;
  return FMC_OK;
}

}  // extern "C"

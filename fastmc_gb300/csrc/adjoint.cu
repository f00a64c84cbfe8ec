// adjoint.cu -- energies of guest snapshots and their adjoints:
// dE/d(guest site coordinates) and dE/d(epsilon, sigma, charge scale) of
// every framework atom type.  No counterpart in the reference.  Two entry
// points: fmc_adjoint_eval_batch, the energy the chains sample (the
// reference's tables, guests with each other too) for a batch of
// snapshots (the `ham_*` kernels, "the sampled Hamiltonian" below), and
// fmc_adjoint_eval, the guest-framework energy of one snapshot with exact
// erfc and analytic Lennard-Jones (the `adj_*` kernels), described here:
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

#include <algorithm>
#include <climits>
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
using fmcdev::rint_image;

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
    n = cap = v.size();
    if (n) {
      FMC_ACUDA(cudaMalloc(&p, n * sizeof(T)));
      FMC_ACUDA(cudaMemcpy(p, v.data(), n * sizeof(T), cudaMemcpyHostToDevice));
    }
  }
  void alloc(size_t count) {
    if (p) cudaFree(p);
    p = nullptr;
    n = cap = count;
    if (n) FMC_ACUDA(cudaMalloc(&p, n * sizeof(T)));
  }
  // grow-only: reallocate only when count exceeds what is held
  void reserve(size_t count) {
    count = std::max<size_t>(count, 1);
    if (count > cap) alloc(count);
    n = count;
  }
  void put(const std::vector<T> &v) {
    reserve(v.size());
    if (!v.empty()) FMC_ACUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  }
  size_t cap = 0;
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


// ------------------------------------------------ the sampled Hamiltonian
// Batched snapshots, the energy the chains sample: the guests' real-space
// erfc Coulomb and Lennard-Jones terms from the reference's tables (erc and
// vvv with the 3-point interpolation, ewald.f:703-715, vdw_terms.f:441-453)
// against the framework and against the other molecules, the reciprocal sum
// of the guests against the framework and the guests (each molecule's own
// |s_m|^2 included), and the guest-framework Lennard-Jones tail (lrcorrect,
// vdw_terms.f:470-645).  Left out are the terms that no coordinate or
// parameter moves: a constant per molecule (the excluded intramolecular
// pairs, ewald3, and the Ewald self energy), the framework's own energy
// (it does move with lambda, but equally in every snapshot) and the
// guest-guest tail.  Framework type t's (eps_t, sigma_t)
// move its pairs' parameters from the FIELD's values as Lorentz-Berthelot
// mixing does (eps x sqrt(eps_t / eps_t0), sigma + (sigma_t - sigma_t0)/2),
// so the tables at the base parameters are the system's own; lambda_t
// scales the type's charges.  Pair terms in T (float or double), sums in
// FP64.  In float, a pair's separation is formed from hi/lo float pairs of
// the two positions (the minimum image taken off exactly), so it carries
// the relative error of one float rounding, as the trial-move path's.

constexpr int kHT = 256;  // threads per block, Hamiltonian kernels
constexpr int kHW = kHT / 32;

struct HamConst {
  double L[3], rL[3];
  float Lh[3], Ll[3], rLf[3];
  double rc2, rengunit, krecip, rdrewd, rdlrpot;
  int mxegrd, tabstride, nfw, ns, ntype, nk, nc[3];
  int kmin[3], kext[3];  // per axis: the smallest k index and the count of indices
  double chgea[kMaxASite], qs[kMaxASite];
  int gg_row[kMaxASite][kMaxASite];  // guest-guest LJ table row, -1 without
  double eps_t[kMaxAType];           // eps_t of the call (FIELD unit), for dE/deps
  double lam[kMaxAType];
  // float copies for the FP32 kernels (no conversion instructions there)
  float rdrewdf, rdlrpotf, rc2f, ncf[3], wf[3], rwf[3];  // wf: cell widths, rwf = 1 / wf
  float chgeaf[kMaxASite], qsf[kMaxASite], lamf[kMaxAType];
};

template <class T>
struct HamT;  // the call's constants in the pair type
template <>
struct HamT<float> {
  static __device__ __forceinline__ float rd(const HamConst &c) { return c.rdrewdf; }
  static __device__ __forceinline__ float rdl(const HamConst &c) { return c.rdlrpotf; }
  static __device__ __forceinline__ float rc2(const HamConst &c) { return c.rc2f; }
  static __device__ __forceinline__ float chgea(const HamConst &c, int s) { return c.chgeaf[s]; }
  static __device__ __forceinline__ float qs(const HamConst &c, int s) { return c.qsf[s]; }
  static __device__ __forceinline__ float lam(const HamConst &c, int t) { return c.lamf[t]; }
};
template <>
struct HamT<double> {
  static __device__ __forceinline__ double rd(const HamConst &c) { return c.rdrewd; }
  static __device__ __forceinline__ double rdl(const HamConst &c) { return c.rdlrpot; }
  static __device__ __forceinline__ double rc2(const HamConst &c) { return c.rc2; }
  static __device__ __forceinline__ double chgea(const HamConst &c, int s) { return c.chgea[s]; }
  static __device__ __forceinline__ double qs(const HamConst &c, int s) { return c.qs[s]; }
  static __device__ __forceinline__ double lam(const HamConst &c, int t) { return c.lam[t]; }
};

// Table position of r: node l and fraction p of the 3-point interpolation
// (false outside the table).  In float, floor(t) comes from adding 2^23
// rounded down (exact for 0 <= t < 2^23) and its bits, with no conversion
// instruction (those issue to the FP64 pipe, which this part has little of).
template <class T>
__device__ __forceinline__ bool tab_pos(T r, T rd, int mx, int &l, T &p) {
  const T t = r * rd;
  if constexpr (sizeof(T) == 4) {
    const float tt = __fadd_rd(t, 8388608.0f);
    l = __float_as_int(tt) - 0x4B000000;
    p = t - (tt - 8388608.0f);
  } else {
    l = int(t);
    p = t - T(l);
  }
  return l >= 1 && l <= mx;
}

// The 3-point interpolation at (l, p), and with interp_d its derivative in r.
template <class T>
__device__ __forceinline__ T interp(const T *tab, int l, T p) {
  const T v0 = tab[l], v1 = tab[l + 1], v2 = tab[l + 2];
  const T t1 = v0 + (v1 - v0) * p;
  const T t2 = v1 + (v2 - v1) * (p - T(1));
  return t1 + (t2 - t1) * p * T(0.5);
}

template <class T>
__device__ __forceinline__ T interp_d(const T *tab, int l, T p, T rd, T &dv) {
  const T v0 = tab[l], v1 = tab[l + 1], v2 = tab[l + 2];
  const T t1 = v0 + (v1 - v0) * p;
  const T t2 = v1 + (v2 - v1) * (p - T(1));
  // d/dp of t1 + (t2 - t1) p / 2, then d/dr = rd d/dp
  dv = ((v1 - v0) + (t2 - t1) * T(0.5) + p * T(0.5) * ((v2 - v1) - (v1 - v0))) * rd;
  return t1 + (t2 - t1) * p * T(0.5);
}

// The interpolant's slope steps at the table's nodes, so the node a pair
// falls on decides its gradient to within that step.  In float, a pair
// within the rounding of r of a node is placed again from its separation
// in FP64, as the FP64 terms place it.
__device__ __forceinline__ bool near_node(float p) { return p < 2e-3f || p > 1.f - 2e-3f; }

template <class T>
__device__ __forceinline__ T warp_sum(T x) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

__device__ __forceinline__ void split_hl(double x, float &h, float &l) {
  h = (float)x;
  l = (float)(x - (double)h);
}

// a - b to the nearest image along one axis, a and b as hi/lo float pairs
// in [0, L): the hi difference with its exact rounding error (two-sum),
// the image taken off the hi part (exact: it is within a factor two of the
// cell edge), then the low parts (|t / L| < 1: rint_image takes the
// nearest integer by comparisons).
__device__ __forceinline__ float mi_hl(float ah, float al, float bh, float bl, float Lh, float Ll,
                                       float rL) {
  const float t = ah - bh;
  const float bb = t - ah;
  const float e = (ah - (t - bb)) + (-bh - bb);
  const float n = rint_image(t * rL);
  return (t - n * Lh) + ((e + (al - bl)) - n * Ll);
}

// One pair's terms: the erfc Coulomb and LJ energies, the LJ sigma
// derivative (framework pairs) and dE/dr / r.  r64 gives the FP64
// separation when a float r lies next to a table node.
template <class T, bool FW, class R64>
__device__ __forceinline__ bool pair_terms(const HamConst &c, T r2, const T *erc, const T *row,
                                           const T *drow, T rd, T rdl, T qq, T lam, R64 &&r64,
                                           T &ev, T &lj, T &dsig, T &f) {
  const T r = sqrt(r2);
  int le, lv;
  T pe, pv;
  bool ine = tab_pos(r, rd, c.mxegrd, le, pe);
  bool inv = tab_pos(r, rdl, c.mxegrd, lv, pv);
  if (sizeof(T) == 4 && (near_node((float)pe) || near_node((float)pv))) {
    const double rr = r64();
    double te = rr * c.rdrewd, tv = rr * c.rdlrpot;
    le = int(te);
    lv = int(tv);
    pe = (T)(te - le);
    pv = (T)(tv - lv);
    ine = le >= 1 && le <= c.mxegrd;
    inv = lv >= 1 && lv <= c.mxegrd;
  }
  T de = T(0), dvv = T(0);
  ev = ine ? interp_d(erc, le, pe, rd, de) : T(0);
  lj = T(0);
  dsig = T(0);
  if (row && inv) {
    lj = interp_d(row, lv, pv, rdl, dvv);
    if (FW) dsig = interp(drow, lv, pv);
  }
  f = (lam * qq * de + dvv) / r;
  return true;
}

// Real space, one block per molecule of the batch.  Framework: the atoms
// are sorted by (type, cell), cells at least rc/2 wide, so that for one
// type the cells of a z-column are one run of atoms.  A warp takes one
// (site, type, half of the 5 x 5 neighbour columns) item at a time; each
// lane sets up one column: skipped when the column lies farther than rc
// from the site in the xy-plane, else the z-cells within the sphere's
// chord, as one run or two where the column wraps in z, each with the
// image the site is shifted by.  The lanes then walk the item's runs as
// one list (each lane stepping from run to run), queue the pairs within
// the cutoff, and evaluate them 32 at a time with one table row and the
// type's sums, which the warp adds to its own shared accumulators.  With
// fewer than five cells a side, one cell holds every atom and each pair
// takes the nearest image.  Guests: threads over the snapshot's other
// molecules, each pair's energy halved (the other molecule's block sees
// it too).  The molecule's site gradients are stored (FP64); the
// snapshot's energy and dE/d(eps, sigma, lambda) per type are added to its
// sums.  T: the type of the pair terms.
constexpr int kColR = 2;                      // neighbour columns each side
constexpr int kNCol = (2 * kColR + 1) * (2 * kColR + 1);
constexpr int kColHalf = (kNCol + 1) / 2;     // columns per item (13, 12)
// cells a side for the column search: a z-chord with its margin spans at
// most 2 kColR + 2 cells, which must not wrap onto itself
constexpr int kFineMin = 2 * kColR + 2;

template <class T>
__global__ void __launch_bounds__(kHT) ham_real_kernel(
    HamConst c, const double4 *__restrict__ fw, const float4 *__restrict__ fwh,
    const float4 *__restrict__ fwl, const int *__restrict__ cstart, const double *__restrict__ xyz,
    const float2 *__restrict__ cw, const int *__restrict__ mol_snap,
    const int *__restrict__ snap_mol0, const int *__restrict__ snap_nmol, const T *__restrict__ erc,
    const T *__restrict__ vt, const T *__restrict__ ds, const T *__restrict__ vgg, double *g64,
    double *esnap, double *psnap) {
  constexpr bool F32 = sizeof(T) == 4;
  __shared__ T acc_p[kHW][kMaxAType][3];  // per warp and type: LJ, dLJ/dsigma, Coulomb / lambda
  __shared__ T acc_g[kHW][kMaxASite][3];  // per warp: site gradients
  __shared__ T acc_e[kHW];                // per warp: guest-guest energy
  __shared__ double site[kMaxASite][3];   // the molecule's sites, wrapped into the cell
  __shared__ float sitef[kMaxASite][6];   // the same as float hi/lo pairs
  __shared__ int sitecell[kMaxASite][3];  // their cells
  __shared__ float rpos[kHW][64][6];      // per warp and run: the shifted site as float hi/lo pairs
  __shared__ signed char rsg[kHW][64][3]; // and the image: site - rsg L
  __shared__ T qprod[kMaxASite][kMaxASite];  // chgea_s q_s2 of guest site pairs
  __shared__ T qv[kHW][4][64];               // per warp: queued pairs (separation, charge)
  __shared__ int qc[kHW][64];                // and (atom index << 6 | run)
  using H = HamT<T>;
  const int m = blockIdx.x, snap = mol_snap[m], ns = c.ns, T_ = c.ntype;
  if (threadIdx.x < kMaxASite * kMaxASite)
    qprod[threadIdx.x / kMaxASite][threadIdx.x % kMaxASite] =
        H::chgea(c, threadIdx.x / kMaxASite) * H::qs(c, threadIdx.x % kMaxASite);
  const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < kHW * kMaxAType * 3; i += kHT) (&acc_p[0][0][0])[i] = T(0);
  for (int i = threadIdx.x; i < kHW * kMaxASite * 3; i += kHT) (&acc_g[0][0][0])[i] = T(0);
  if (threadIdx.x < kHW) acc_e[threadIdx.x] = T(0);
  if (threadIdx.x < 3 * ns) {
    const int d = threadIdx.x % 3;
    const double x = xyz[(size_t)m * ns * 3 + threadIdx.x];
    double w = x - c.L[d] * floor(x * c.rL[d]);
    // a coordinate that is not finite, or so large that the wrap leaves the
    // cell, gives a meaningless energy but no index outside the cell lists
    if (!(w >= 0.0 && w <= c.L[d])) w = 0.0;
    site[threadIdx.x / 3][d] = w;
    sitecell[threadIdx.x / 3][d] = max(0, min(c.nc[d] - 1, (int)(w * c.rL[d] * c.nc[d])));
    split_hl(w, sitef[threadIdx.x / 3][2 * d], sitef[threadIdx.x / 3][2 * d + 1]);
  }
  __syncthreads();
  const bool fine = c.nc[0] >= kFineMin && c.nc[1] >= kFineMin && c.nc[2] >= kFineMin;
  const T rd = H::rd(c), rdl = H::rdl(c), rc2 = H::rc2(c);
  const int ncell = c.nc[0] * c.nc[1] * c.nc[2];
  const int nitem = ns * T_ * (fine ? 2 : 1);
  for (int it = wq; it < nitem; it += kHW) {  // one (site, type, half of the columns) item per warp
    const int half = fine ? it % 2 : 0, st = fine ? it / 2 : it;
    const int t = st % T_, s = st / T_;
    // lane k: column c0 + k (fine) or, lane 0, the one cell (brute force);
    // up to two runs: (first atom, count) each
    int f1 = 0, n1 = 0, f2 = 0, n2 = 0;
    if (fine) {
      const int col = half * kColHalf + lane;
      if (lane < (half ? kNCol - kColHalf : kColHalf)) {
        const int dx = col / (2 * kColR + 1) - kColR, dy = col % (2 * kColR + 1) - kColR;
        const int icx = sitecell[s][0] + dx, icy = sitecell[s][1] + dy;
        // distance in the xy-plane from the site to the column (unwrapped
        // frame), in float with a margin: a column kept needlessly only
        // adds candidates the cutoff test drops
        const float sx = sitef[s][0], sy = sitef[s][2], sz = sitef[s][4];
        const float ex = fmaxf(0.f, fmaxf((float)icx * c.wf[0] - sx, sx - (float)(icx + 1) * c.wf[0]));
        const float ey = fmaxf(0.f, fmaxf((float)icy * c.wf[1] - sy, sy - (float)(icy + 1) * c.wf[1]));
        const float d2 = ex * ex + ey * ey;
        if (d2 < c.rc2f + 1e-2f) {
          const float zh = sqrtf(fmaxf(c.rc2f - d2, 0.f)) + 1e-2f;
          int iz0 = (int)floorf((sz - zh) * c.rwf[2]), iz1 = (int)floorf((sz + zh) * c.rwf[2]);
          iz1 = min(iz1, iz0 + c.nc[2] - 1);
          int ix = icx, iy = icy, sgx = 0, sgy = 0;
          if (ix < 0) { ix += c.nc[0]; sgx = -1; } else if (ix >= c.nc[0]) { ix -= c.nc[0]; sgx = 1; }
          if (iy < 0) { iy += c.nc[1]; sgy = -1; } else if (iy >= c.nc[1]) { iy -= c.nc[1]; sgy = 1; }
          const int cb = (ix * c.nc[1] + iy) * c.nc[2], tb = t * ncell;
          // run 1: the cells inside [0, nz); run 2: the part that wraps
          const int a0 = max(iz0, 0), a1 = min(iz1, c.nc[2] - 1);
          int b0 = 0, b1 = -1, sgz = 0;
          if (iz0 < 0) {
            b0 = iz0 + c.nc[2];
            b1 = c.nc[2] - 1;
            sgz = -1;
          } else if (iz1 >= c.nc[2]) {
            b0 = 0;
            b1 = iz1 - c.nc[2];
            sgz = 1;
          }
          if (a0 <= a1) {
            f1 = cstart[tb + cb + a0];
            n1 = cstart[tb + cb + a1 + 1] - f1;
          }
          if (b0 <= b1) {
            f2 = cstart[tb + cb + b0];
            n2 = cstart[tb + cb + b1 + 1] - f2;
          }
          const int sg[2][3] = {{sgx, sgy, 0}, {sgx, sgy, sgz}};
          for (int r = 0; r < 2; ++r) {
            for (int d = 0; d < 3; ++d) {
              rsg[wq][2 * lane + r][d] = (signed char)sg[r][d];
              // (h + l) - sg L as a hi/lo pair: two-sum of the hi parts, then the lows
              const float h = sitef[s][2 * d], l = sitef[s][2 * d + 1];
              const float bh = -(float)sg[r][d] * c.Lh[d], bl = -(float)sg[r][d] * c.Ll[d];
              const float t0 = h + bh, bb = t0 - h;
              const float e = (h - (t0 - bb)) + (bh - bb);
              const float lo = e + (l + bl);
              const float hi = t0 + lo;
              rpos[wq][2 * lane + r][2 * d] = hi;
              rpos[wq][2 * lane + r][2 * d + 1] = lo - (hi - t0);
            }
          }
        }
      }
    } else if (lane == 0) {
      f1 = cstart[t * ncell];
      n1 = cstart[t * ncell + ncell] - f1;
      for (int d = 0; d < 3; ++d) {
        rsg[wq][0][d] = 0;
        rpos[wq][0][2 * d] = sitef[s][2 * d];
        rpos[wq][0][2 * d + 1] = sitef[s][2 * d + 1];
      }
    }
    const int cnt = n1 + n2;
    int incl = cnt;  // inclusive scan of the lanes' counts
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    __syncwarp();
    if (total == 0) continue;
    const T *row = vt + ((size_t)s * T_ + t) * c.tabstride;
    const T *drow = ds + ((size_t)s * T_ + t) * c.tabstride;
    const T ca = H::chgea(c, s), lam = H::lam(c, t);
    T plj = 0, pds = 0, pco = 0, gx = 0, gy = 0, gz = 0;
    // pairs within the cutoff wait in the warp's queue; 32 at a time, one
    // per lane, take the table terms
    auto run_pairs = [&](int n) {
      __syncwarp();
      if (lane < n) {
        const int code = qc[wq][lane], j = code >> 6, rr = code & 63;
        const T dx = qv[wq][0][lane], dy = qv[wq][1][lane], dz = qv[wq][2][lane], qa = qv[wq][3][lane];
        T ev, lj, dsig, f;
        pair_terms<T, true>(c, dx * dx + dy * dy + dz * dz, erc, row, drow, rd, rdl, ca * qa, lam,
                            [&]() {
                              const double4 a = fw[j];
                              double ex = site[s][0] - rsg[wq][rr][0] * c.L[0] - a.x;
                              double ey = site[s][1] - rsg[wq][rr][1] * c.L[1] - a.y;
                              double ez = site[s][2] - rsg[wq][rr][2] * c.L[2] - a.z;
                              if (!fine) {
                                ex -= c.L[0] * rint(ex * c.rL[0]);
                                ey -= c.L[1] * rint(ey * c.rL[1]);
                                ez -= c.L[2] * rint(ez * c.rL[2]);
                              }
                              return sqrt(ex * ex + ey * ey + ez * ez);
                            },
                            ev, lj, dsig, f);
        gx += f * dx;
        gy += f * dy;
        gz += f * dz;
        plj += lj;
        pds += dsig;
        pco += ca * qa * ev;
      }
      __syncwarp();
    };
    int qn = 0;                    // queued pairs (warp-uniform)
    int k = -1, end = 0, mid = 0;  // this lane's column, its list end and the end of its first run
    int o1 = 0, o2 = 0;            // atom index = list index + offset, per run
    int rr = 0;                    // the run (2 k + 0 or 1)
    float xh = 0.f, xl = 0.f, yh = 0.f, yl = 0.f, zh = 0.f, zl = 0.f;
    double px = 0.0, py = 0.0, pz = 0.0;
    const int excl = incl - cnt;
    for (int base = 0; base < total; base += 32) {
      const int idx = base + lane;
      const bool act = idx < total;
      while (__any_sync(0xffffffffu, act && idx >= end)) {  // step to the column holding idx
        const int nk = k + 1;
        const int ne = __shfl_sync(0xffffffffu, incl, nk & 31);
        const int nx = __shfl_sync(0xffffffffu, excl, nk & 31);
        const int nn1 = __shfl_sync(0xffffffffu, n1, nk & 31);
        const int nf1 = __shfl_sync(0xffffffffu, f1, nk & 31);
        const int nf2 = __shfl_sync(0xffffffffu, f2, nk & 31);
        if (act && idx >= end) {
          k = nk;
          end = ne;
          mid = nx + nn1;
          o1 = nf1 - nx;
          o2 = nf2 - mid;
        }
      }
      int j = 0;
      if (act) {
        const int r = idx < mid ? 0 : 1;
        j = idx + (r == 0 ? o1 : o2);
        const int nr = 2 * k + r;
        if (nr != rr || base == 0) {  // the site shifted by this run's image
          rr = nr;
          xh = rpos[wq][rr][0];
          xl = rpos[wq][rr][1];
          yh = rpos[wq][rr][2];
          yl = rpos[wq][rr][3];
          zh = rpos[wq][rr][4];
          zl = rpos[wq][rr][5];
          if (!F32 || !fine) {
            px = site[s][0] - rsg[wq][rr][0] * c.L[0];
            py = site[s][1] - rsg[wq][rr][1] * c.L[1];
            pz = site[s][2] - rsg[wq][rr][2] * c.L[2];
          }
        }
      }
      T dx = T(0), dy = T(0), dz = T(0), qa = T(0);
      if (act) {
        if (F32 && fine) {
          const float4 ah = fwh[j], al = fwl[j];
          dx = (T)((xh - ah.x) + (xl - al.x));
          dy = (T)((yh - ah.y) + (yl - al.y));
          dz = (T)((zh - ah.z) + (zl - al.z));
          qa = (T)ah.w;
        } else {
          const double4 a = fw[j];
          double ex = px - a.x, ey = py - a.y, ez = pz - a.z;
          if (!fine) {
            ex -= c.L[0] * rint(ex * c.rL[0]);
            ey -= c.L[1] * rint(ey * c.rL[1]);
            ez -= c.L[2] * rint(ez * c.rL[2]);
          }
          dx = (T)ex;
          dy = (T)ey;
          dz = (T)ez;
          qa = (T)a.w;
        }
      }
      const bool in = act && dx * dx + dy * dy + dz * dz < rc2;
      const unsigned bm = __ballot_sync(0xffffffffu, in);
      if (in) {
        const int pos = qn + __popc(bm & ((1u << lane) - 1u));
        qv[wq][0][pos] = dx;
        qv[wq][1][pos] = dy;
        qv[wq][2][pos] = dz;
        qv[wq][3][pos] = qa;
        qc[wq][pos] = (j << 6) | rr;
      }
      qn += __popc(bm);
      if (qn >= 32) {
        run_pairs(32);
        if (lane < qn - 32) {
          for (int d = 0; d < 4; ++d) qv[wq][d][lane] = qv[wq][d][32 + lane];
          qc[wq][lane] = qc[wq][32 + lane];
        }
        qn -= 32;
      }
    }
    if (qn > 0) run_pairs(qn);
    plj = warp_sum(plj);
    pds = warp_sum(pds);
    pco = warp_sum(pco);
    gx = warp_sum(gx);
    gy = warp_sum(gy);
    gz = warp_sum(gz);
    if (lane == 0) {
      acc_p[wq][t][0] += plj;
      acc_p[wq][t][1] += pds;
      acc_p[wq][t][2] += pco;
      acc_g[wq][s][0] += gx;
      acc_g[wq][s][1] += gy;
      acc_g[wq][s][2] += gz;
    }
    __syncwarp();
  }
  // the snapshot's other molecules, one site of this molecule at a time;
  // pairs within the cutoff queued per warp as for the framework
  {
    const int m0 = snap_mol0[snap], nm = snap_nmol[snap];
    T pe = 0;
    for (int s = 0; s < ns; ++s) {
      float sh[3] = {0.f, 0.f, 0.f}, sl[3] = {0.f, 0.f, 0.f};
      if (F32)
        for (int d = 0; d < 3; ++d) {
          const float2 v = cw[((size_t)m * ns + s) * 3 + d];
          sh[d] = v.x;
          sl[d] = v.y;
        }
      T gx = 0, gy = 0, gz = 0;
      auto run_pairs = [&](int n) {
        __syncwarp();
        if (lane < n) {
          const int code = qc[wq][lane], s2 = code & 7;
          const size_t i2 = (size_t)(code >> 3) * ns + s2;
          const T dx = qv[wq][0][lane], dy = qv[wq][1][lane], dz = qv[wq][2][lane];
          const int rowi = c.gg_row[s][s2];
          const T qq = qprod[s][s2];
          T ev, lj, dsig, f;
          pair_terms<T, false>(c, dx * dx + dy * dy + dz * dz, erc,
                               rowi >= 0 ? vgg + (size_t)rowi * c.tabstride : nullptr, nullptr, rd, rdl, qq,
                               T(1),
                               [&]() {
                                 double ex = site[s][0] - xyz[3 * i2], ey = site[s][1] - xyz[3 * i2 + 1],
                                        ez = site[s][2] - xyz[3 * i2 + 2];
                                 ex -= c.L[0] * rint(ex * c.rL[0]);
                                 ey -= c.L[1] * rint(ey * c.rL[1]);
                                 ez -= c.L[2] * rint(ez * c.rL[2]);
                                 return sqrt(ex * ex + ey * ey + ez * ez);
                               },
                               ev, lj, dsig, f);
          gx += f * dx;
          gy += f * dy;
          gz += f * dz;
          pe += T(0.5) * (qq * ev + lj);
        }
        __syncwarp();
      };
      int qn = 0;
      for (int mb = m0 + 32 * wq; mb < m0 + nm; mb += kHT) {
        const int mm = mb + lane;
        const bool act = mm < m0 + nm && mm != m;
        for (int s2 = 0; s2 < ns; ++s2) {
          const size_t i2 = (size_t)mm * ns + s2;
          T dx = T(0), dy = T(0), dz = T(0);
          if (act) {
            if (F32) {
              const float2 qx = cw[3 * i2], qy = cw[3 * i2 + 1], qz = cw[3 * i2 + 2];
              dx = (T)mi_hl(sh[0], sl[0], qx.x, qx.y, c.Lh[0], c.Ll[0], c.rLf[0]);
              dy = (T)mi_hl(sh[1], sl[1], qy.x, qy.y, c.Lh[1], c.Ll[1], c.rLf[1]);
              dz = (T)mi_hl(sh[2], sl[2], qz.x, qz.y, c.Lh[2], c.Ll[2], c.rLf[2]);
            } else {
              double ex = site[s][0] - xyz[3 * i2], ey = site[s][1] - xyz[3 * i2 + 1],
                     ez = site[s][2] - xyz[3 * i2 + 2];
              ex -= c.L[0] * rint(ex * c.rL[0]);
              ey -= c.L[1] * rint(ey * c.rL[1]);
              ez -= c.L[2] * rint(ez * c.rL[2]);
              dx = (T)ex;
              dy = (T)ey;
              dz = (T)ez;
            }
          }
          const bool in = act && dx * dx + dy * dy + dz * dz < rc2;
          const unsigned bm = __ballot_sync(0xffffffffu, in);
          if (in) {
            const int pos = qn + __popc(bm & ((1u << lane) - 1u));
            qv[wq][0][pos] = dx;
            qv[wq][1][pos] = dy;
            qv[wq][2][pos] = dz;
            qc[wq][pos] = (mm << 3) | s2;
          }
          qn += __popc(bm);
          if (qn >= 32) {
            run_pairs(32);
            if (lane < qn - 32) {
              for (int d = 0; d < 3; ++d) qv[wq][d][lane] = qv[wq][d][32 + lane];
              qc[wq][lane] = qc[wq][32 + lane];
            }
            qn -= 32;
          }
        }
      }
      if (qn > 0) run_pairs(qn);
      gx = warp_sum(gx);
      gy = warp_sum(gy);
      gz = warp_sum(gz);
      if (lane == 0) {
        acc_g[wq][s][0] += gx;
        acc_g[wq][s][1] += gy;
        acc_g[wq][s][2] += gz;
      }
    }
    pe = warp_sum(pe);
    if (lane == 0) acc_e[wq] += pe;
  }
  __syncthreads();
  // the warps' sums in FP64: site gradients, and per type dE/d(eps, sigma,
  // lambda) and the energy (warp 0; the types are at most 16)
  if (threadIdx.x < 3 * ns) {
    const int s = threadIdx.x / 3, d = threadIdx.x % 3;
    double g = 0.0;
    for (int w = 0; w < kHW; ++w) g += (double)acc_g[w][s][d];
    g64[(size_t)m * ns * 3 + threadIdx.x] = g * c.rengunit;
  }
  if (wq == 0) {
    double e = 0.0;
    if (lane < T_) {
      const int t = lane;
      double lj = 0.0, dsg = 0.0, co = 0.0;
      for (int w = 0; w < kHW; ++w) {
        lj += (double)acc_p[w][t][0];
        dsg += (double)acc_p[w][t][1];
        co += (double)acc_p[w][t][2];
      }
      double *p = psnap + (size_t)snap * 3 * T_ + 3 * t;
      if (c.eps_t[t] > 0.0 && lj != 0.0) atomicAdd(p, lj / (2.0 * c.eps_t[t]) * c.rengunit);
      if (dsg != 0.0) atomicAdd(p + 1, dsg * c.rengunit);
      if (co != 0.0) atomicAdd(p + 2, co * c.rengunit);
      e = c.lam[t] * co + lj;
    }
    if (lane < kHW) e += (double)acc_e[lane];
    e = warp_sum(e);
    if (lane == 0 && e != 0.0) atomicAdd(esnap + snap, e * c.rengunit);
  }
}

// Per site: fractional coordinates x / L reduced to [0, 1) and the
// Cartesian position wrapped into [0, L), both as float hi/lo pairs.
__global__ void ham_frac_kernel(HamConst c, const double *xyz, int nsite, float2 *fr, float2 *cw) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * nsite) return;
  const int d = i % 3;
  double f = xyz[i] * c.rL[d];
  f -= floor(f);
  float h, l;
  split_hl(f, h, l);
  fr[i] = make_float2(h, l);
  split_hl(xyz[i] - c.L[d] * floor(xyz[i] * c.rL[d]), h, l);
  cw[i] = make_float2(h, l);
}

// e^{i 2 pi (l fx + m fy + n fz)} of one site: FP64, or in FP32 with the
// products j * f formed exactly (FMA residuals) and reduced before sincospif.
template <class T>
__device__ __forceinline__ void ham_phase(const int4 l, const double *xyz, const float2 *fr, double rLx,
                                          double rLy, double rLz, T &cs, T &sn) {
  if constexpr (sizeof(T) == 8) {
    double f = (double)l.x * (xyz[0] * rLx) + (double)l.y * (xyz[1] * rLy) + (double)l.z * (xyz[2] * rLz);
    f -= rint(f);
    sincospi(2.0 * f, &sn, &cs);
  } else {
    float hs = 0.f, ls = 0.f;
    const int lk[3] = {l.x, l.y, l.z};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const float j = (float)lk[d];
      const float p = j * fr[d].x;
      const float pe = fmaf(j, fr[d].x, -p) + j * fr[d].y;
      const float t = hs + p;
      const float bp = t - hs;
      ls += ((hs - (t - bp)) + (p - bp)) + pe;
      hs = t;
    }
    float x = (hs - rintf(hs)) + ls;
    sincospif(2.0f * x, &sn, &cs);
  }
}

// The guests' structure factor of every snapshot (block x), k per thread: S_g, and
// the reciprocal energy K a_k [2 Re(S_g conj(S_fw)) + |S_g|^2] with S_fw =
// sum_t lambda_t S_t, dE/dlambda_t = K a_k 2 Re(S_g conj(S_t)).  |S_g|^2
// keeps each molecule's own |s_m|^2: it depends on the orientation (a
// finite k set), and the reference's insertion energy carries it.
template <class T>
__global__ void __launch_bounds__(kHT) ham_sk_kernel(HamConst c, const int4 *__restrict__ klmn,
                                                     const double *__restrict__ akk,
                                                     const double2 *__restrict__ skt,
                                                     const double *__restrict__ xyz,
                                                     const float2 *__restrict__ fr,
                                                     const int *__restrict__ snap_mol0,
                                                     const int *__restrict__ snap_nmol, double2 *sg,
                                                     double *esnap, double *psnap) {
  constexpr int NV = 1 + 3 * kMaxAType;
  __shared__ double sh[(kHT / 32) * NV];
  const int k = blockIdx.y * kHT + threadIdx.x, snap = blockIdx.x, ns = c.ns;
  double v[NV];
  for (int q = 0; q < NV; ++q) v[q] = 0.0;
  if (k < c.nk) {
    const int4 l = klmn[k];
    double Sr = 0.0, Si = 0.0;
    const int m0 = snap_mol0[snap], nm = snap_nmol[snap];
    for (int mm = m0; mm < m0 + nm; ++mm) {
      T sr = T(0), si = T(0);  // one molecule in T, the snapshot's sum in FP64
      for (int s = 0; s < ns; ++s) {
        const size_t i = (size_t)mm * ns + s;
        T cs, sn;
        ham_phase<T>(l, xyz + 3 * i, fr + 3 * i, c.rL[0], c.rL[1], c.rL[2], cs, sn);
        sr += (T)c.qs[s] * cs;
        si += (T)c.qs[s] * sn;
      }
      Sr += (double)sr;
      Si += (double)si;
    }
    double Fr = 0.0, Fi = 0.0;
    const double f = c.krecip * akk[k] * c.rengunit;
    for (int t = 0; t < c.ntype; ++t) {
      const double2 st = skt[(size_t)t * c.nk + k];
      Fr += c.lam[t] * st.x;
      Fi += c.lam[t] * st.y;
      v[1 + 3 * t + 2] = 2.0 * f * (Sr * st.x + Si * st.y);
    }
    v[0] = f * (2.0 * (Sr * Fr + Si * Fi) + (Sr * Sr + Si * Si));
    sg[(size_t)snap * c.nk + k] = make_double2(Sr + Fr, Si + Fi);  // S_g + S_fw
  }
  const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
  const int nv = 1 + 3 * c.ntype;
  for (int i = 0; i < nv; ++i) {
    double x = v[i];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[wq * NV + i] = x;
  }
  __syncthreads();
  if (threadIdx.x < nv) {
    double t = 0.0;
    for (int q = 0; q < kHT / 32; ++q) t += sh[q * NV + threadIdx.x];
    if (t != 0.0) atomicAdd(threadIdx.x == 0 ? esnap + snap : psnap + (size_t)snap * 3 * c.ntype + threadIdx.x - 1, t);
  }
}

// e^{i 2 pi j f} for one axis, f a hi/lo fraction in [0, 1): j f formed
// exactly (FMA residual) and reduced before sincospif.
__device__ __forceinline__ float2 axis_phase(float jf, float2 f) {
  const float p = jf * f.x;
  const float pe = fmaf(jf, f.x, -p) + jf * f.y;
  const float x = (p - rintf(p)) + pe;
  float sn, cs;
  sincospif(2.0f * x, &sn, &cs);
  return make_float2(cs, sn);
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// The guests' structure factor in FP32 (block: one snapshot and 256
// k-vectors): the snapshot's sites in runs of whole molecules, each run's
// per-axis phase tables e^{i 2 pi j f_d} built once in shared memory, so a
// thread's phase at k = (l, m, n) is the product of three table entries.
// Molecule sums in float, the snapshot's in FP64; then as ham_sk_kernel.
constexpr int kSkRun = 64;  // sites per table run at most

__global__ void __launch_bounds__(kHT) ham_sk32_kernel(HamConst c, const int4 *__restrict__ klmn,
                                                       const double *__restrict__ akk,
                                                       const double2 *__restrict__ skt,
                                                       const float2 *__restrict__ fr,
                                                       const int *__restrict__ snap_mol0,
                                                       const int *__restrict__ snap_nmol, double2 *sg,
                                                       float2 *sgf, double *esnap, double *psnap) {
  extern __shared__ float2 ptab[];  // [site of the run][KX + KY + KZ]
  constexpr int NV = 1 + 3 * kMaxAType;
  __shared__ double sh[(kHT / 32) * NV];
  const int KX = c.kext[0], KY = c.kext[1], KW = c.kext[0] + c.kext[1] + c.kext[2];
  const int k = blockIdx.y * kHT + threadIdx.x, snap = blockIdx.x, ns = c.ns;
  int ix = 0, iy = 0, iz = 0;
  if (k < c.nk) {
    const int4 l = klmn[k];
    ix = l.x - c.kmin[0];
    iy = KX + l.y - c.kmin[1];
    iz = KX + KY + l.z - c.kmin[2];
  }
  float qs[kMaxASite];
#pragma unroll
  for (int s = 0; s < kMaxASite; ++s) qs[s] = s < ns ? (float)c.qs[s] : 0.f;
  const int m0 = snap_mol0[snap], nm = snap_nmol[snap];
  const int mrun = max(1, kSkRun / ns);  // molecules per run
  double Sr = 0.0, Si = 0.0;
  for (int r0 = 0; r0 < nm; r0 += mrun) {
    const int nr = min(mrun, nm - r0), nsite = nr * ns;
    const size_t site0 = (size_t)(m0 + r0) * ns;
    __syncthreads();
    for (int e = threadIdx.x; e < nsite * KW; e += kHT) {
      const int si = e / KW, w = e % KW;
      const int d = w < KX ? 0 : (w < KX + KY ? 1 : 2);
      const int j = d == 0 ? w + c.kmin[0] : (d == 1 ? w - KX + c.kmin[1] : w - KX - KY + c.kmin[2]);
      ptab[e] = axis_phase((float)j, fr[(site0 + si) * 3 + d]);
    }
    __syncthreads();
    if (k < c.nk) {
      float rr = 0.f, ri = 0.f;  // the run's sum in float, the snapshot's in FP64
      for (int mm = 0; mm < nr; ++mm) {
#pragma unroll
        for (int s = 0; s < kMaxASite; ++s) {
          if (s >= ns) break;
          const float2 *t = ptab + (mm * ns + s) * KW;
          const float2 e = cmul(cmul(t[ix], t[iy]), t[iz]);
          rr += qs[s] * e.x;
          ri += qs[s] * e.y;
        }
      }
      Sr += (double)rr;
      Si += (double)ri;
    }
  }
  // the reciprocal energy and dE/dlambda_t, reduced over the block
  const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
  const double f = k < c.nk ? c.krecip * akk[k] * c.rengunit : 0.0;
  double Fr = 0.0, Fi = 0.0;
  for (int t = 0; t < c.ntype; ++t) {
    double dl = 0.0;
    if (k < c.nk) {
      const double2 st = skt[(size_t)t * c.nk + k];
      Fr += c.lam[t] * st.x;
      Fi += c.lam[t] * st.y;
      dl = 2.0 * f * (Sr * st.x + Si * st.y);
    }
    dl = warp_sum(dl);
    if (lane == 0) sh[wq * NV + 1 + t] = dl;
  }
  double e = 0.0;
  if (k < c.nk) {
    e = f * (2.0 * (Sr * Fr + Si * Fi) + (Sr * Sr + Si * Si));
    sg[(size_t)snap * c.nk + k] = make_double2(Sr + Fr, Si + Fi);  // S_g + S_fw
    sgf[(size_t)snap * c.nk + k] = make_float2((float)(Sr + Fr), (float)(Si + Fi));
  }
  e = warp_sum(e);
  if (lane == 0) sh[wq * NV] = e;
  __syncthreads();
  if (threadIdx.x <= c.ntype) {
    double t = 0.0;
    for (int q = 0; q < kHT / 32; ++q) t += sh[q * NV + threadIdx.x];
    if (t != 0.0)
      atomicAdd(threadIdx.x == 0 ? esnap + snap : psnap + (size_t)snap * 3 * c.ntype + 3 * (threadIdx.x - 1) + 2, t);
  }
}

inline size_t ham_sk32_smem(const HamConst &h) {
  return sizeof(float2) * (size_t)std::max(1, kSkRun / h.ns) * h.ns * (h.kext[0] + h.kext[1] + h.kext[2]);
}

// Reciprocal site gradients in FP32, one thread per molecule, k in the
// list's order: along a row of n (same l and m, n one more) a site's phase
// steps by e^{i 2 pi f_z}; it is formed anew at each row's start and after
// every 8 steps.  Otherwise as ham_recip_grad_kernel.
template <int NS>
__global__ void ham_recip_grad32_kernel(HamConst c, const int4 *__restrict__ klmn,
                                        const float4 *__restrict__ klf, const float4 *__restrict__ kv,
                                        const float2 *__restrict__ sg, const float2 *__restrict__ fr,
                                        const int *__restrict__ mol_snap, int nmol_total,
                                        const double *__restrict__ g64, float *gout) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nmol_total) return;
  const int ns = c.ns, snap = mol_snap[m];
  double g[NS][3];
  float gc[NS][3], qs[NS];
  float2 ph[NS], ez[NS];
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    g[s][0] = g[s][1] = g[s][2] = 0.0;
    gc[s][0] = gc[s][1] = gc[s][2] = 0.f;
    qs[s] = s < ns ? (float)c.qs[s] : 0.f;
    ez[s] = s < ns ? axis_phase(1.f, fr[((size_t)m * ns + s) * 3 + 2]) : make_float2(1.f, 0.f);
    ph[s] = make_float2(1.f, 0.f);
  }
  const float2 *w = sg + (size_t)snap * c.nk;
  int4 prev = make_int4(INT_MIN, 0, 0, 0);
  int steps = 0;
  for (int k = 0; k < c.nk; ++k) {
    const int4 l = klmn[k];
    const bool step = l.x == prev.x && l.y == prev.y && l.z == prev.z + 1 && steps < 8;
    steps = step ? steps + 1 : 0;
    prev = l;
    const float4 kk = kv[k];
    const float2 w0 = w[k];
    const float wr = w0.x, wi = w0.y, f = kk.w, kx = kk.x, ky = kk.y, kz = kk.z;
    float4 lf = make_float4(0.f, 0.f, 0.f, 0.f);
    if (!step) lf = klf[k];
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      if (NS == kMaxASite && s >= ns) break;
      if (step) {
        ph[s] = cmul(ph[s], ez[s]);
      } else {
        const float2 *q = fr + ((size_t)m * ns + s) * 3;
        ph[s] = cmul(cmul(axis_phase(lf.x, q[0]), axis_phase(lf.y, q[1])), axis_phase(lf.z, q[2]));
      }
      const float a = f * qs[s] * (ph[s].y * wr - ph[s].x * wi);
      gc[s][0] += a * kx;
      gc[s][1] += a * ky;
      gc[s][2] += a * kz;
    }
    if ((k & 31) == 31 || k == c.nk - 1) {
#pragma unroll
      for (int s = 0; s < NS; ++s)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          g[s][d] += (double)gc[s][d];
          gc[s][d] = 0.f;
        }
    }
  }
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    if (NS == kMaxASite && s >= ns) break;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const size_t i = ((size_t)m * ns + s) * 3 + d;
      gout[i] = (float)(g64[i] + g[s][d] * c.rengunit);
    }
  }
}

// Reciprocal site gradients, one thread per molecule: dE/dr_i = -2 K q_i
// sum_k a_k k Im(e^{i phi_i} conj(W)), W = S_fw + S_g, with kv[k] = (k,
// -2 K a_k); in T, summed in T over runs of 32 k-vectors and those in
// FP64; added to the real-space gradients and stored as float (3N x FP32).
template <class T>
__global__ void ham_recip_grad_kernel(HamConst c, const int4 *__restrict__ klmn,
                                      const double4 *__restrict__ kv, const double2 *__restrict__ sg,
                                      const double *__restrict__ xyz, const float2 *__restrict__ fr,
                                      const int *__restrict__ mol_snap, int nmol_total,
                                      const double *__restrict__ g64, float *gout) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nmol_total) return;
  const int ns = c.ns, snap = mol_snap[m];
  double g[kMaxASite][3];
  T gc[kMaxASite][3];
  T qs[kMaxASite];
#pragma unroll
  for (int s = 0; s < kMaxASite; ++s) {
    g[s][0] = g[s][1] = g[s][2] = 0.0;
    gc[s][0] = gc[s][1] = gc[s][2] = T(0);
    qs[s] = s < ns ? (T)c.qs[s] : T(0);
  }
  const double2 *w = sg + (size_t)snap * c.nk;
  for (int k = 0; k < c.nk; ++k) {
    const int4 l = klmn[k];
    const double4 kk = kv[k];
    const double2 w0 = w[k];
    const T wr = (T)w0.x, wi = (T)w0.y, f = (T)kk.w, kx = (T)kk.x, ky = (T)kk.y, kz = (T)kk.z;
#pragma unroll
    for (int s = 0; s < kMaxASite; ++s) {
      if (s >= ns) break;
      const size_t i = (size_t)m * ns + s;
      T cs, sn;
      ham_phase<T>(l, xyz + 3 * i, fr + 3 * i, c.rL[0], c.rL[1], c.rL[2], cs, sn);
      const T a = f * qs[s] * (sn * wr - cs * wi);
      gc[s][0] += a * kx;
      gc[s][1] += a * ky;
      gc[s][2] += a * kz;
    }
    if ((k & 31) == 31 || k == c.nk - 1) {
#pragma unroll
      for (int s = 0; s < kMaxASite; ++s)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          g[s][d] += (double)gc[s][d];
          gc[s][d] = T(0);
        }
    }
  }
#pragma unroll
  for (int s = 0; s < kMaxASite; ++s) {
    if (s >= ns) break;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const size_t i = ((size_t)m * ns + s) * 3 + d;
      gout[i] = (float)(g64[i] + g[s][d] * c.rengunit);
    }
  }
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
  // the sampled Hamiltonian (fmc_adjoint_eval_batch)
  HamConst h{};
  ABuf<double4> hfw;         // framework atoms sorted by (cell, type), wrapped into the cell, charge
  ABuf<float4> hfwh, hfwl;   // the same positions as float hi/lo pairs (hi carries the charge)
  ABuf<int> hcstart;         // [type * ncell + cell] first atom, ntype * ncell + 1 entries
  ABuf<double4> kv;          // per k-vector: (k, -2 krecip a_k)
  ABuf<float4> kv32, klf;    // the same in float, and (l, m, n) as floats
  ABuf<double> erc64, vgg64;
  ABuf<float> erc32, vgg32;
  std::vector<double> eps0, sig0;  // [site][type] the FIELD's pair parameters (internal unit, A)
  std::vector<double> ntyp;        // framework atoms per type
  double volm = 0, rcut = 0, engunit = 1, dlrpot = 0;
  // per-call buffers, kept between calls and grown when a batch needs more
  struct Scratch {
    ABuf<int> dms, dm0, dnm;
    ABuf<double> e_d, p_d, g64, vt64, ds64;
    ABuf<float> vt32, ds32;
    ABuf<float2> fr, cw, sgf;
    ABuf<double2> sg;
  } w;
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
    if (c.nfw >= (1 << 25)) raise(FMC_ERR_CAPACITY, "the adjoint takes fewer than 2^25 framework atoms");
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
    // the sampled Hamiltonian: tables, framework cells, pair parameters
    HamConst &h = a->h;
    for (int d = 0; d < 3; ++d) {
      h.L[d] = c.L[d];
      h.rL[d] = c.rL[d];
      h.Lh[d] = (float)c.L[d];
      h.Ll[d] = (float)(c.L[d] - (double)h.Lh[d]);
      h.rLf[d] = (float)c.rL[d];
      h.nc[d] = (int)std::floor(c.L[d] / (0.5 * s.rcut));  // cells at least rc / 2 wide
    }
    if (h.nc[0] < kFineMin || h.nc[1] < kFineMin || h.nc[2] < kFineMin)
      h.nc[0] = h.nc[1] = h.nc[2] = 1;  // small cells: one cell, every atom, nearest image per pair
    for (int d = 0; d < 3; ++d) {
      h.wf[d] = (float)(c.L[d] / h.nc[d]);
      h.rwf[d] = (float)(h.nc[d] / c.L[d]);
    }
    if (2.0 * s.rcut > std::min(c.L[0], std::min(c.L[1], c.L[2])))
      raise(FMC_ERR_INPUT, "the adjoint needs the cutoff below half the cell");
    h.rc2 = c.rc2;
    h.rengunit = c.rengunit;
    h.krecip = c.krecip;
    h.rdrewd = 1.0 / s.drewd;
    h.rdlrpot = 1.0 / s.dlrpot;
    h.mxegrd = s.mxegrd;
    h.tabstride = s.mxegrd + 3;
    h.rdrewdf = (float)h.rdrewd;
    h.rdlrpotf = (float)h.rdlrpot;
    h.rc2f = (float)h.rc2;
    for (int d = 0; d < 3; ++d) h.ncf[d] = (float)h.nc[d];
    {
      int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
      for (int k = 0; k < s.newld; ++k) {
        const int v[3] = {s.kl[k], s.km[k], s.kn[k]};
        for (int d = 0; d < 3; ++d) {
          lo[d] = std::min(lo[d], v[d]);
          hi[d] = std::max(hi[d], v[d]);
        }
      }
      for (int d = 0; d < 3; ++d) {
        h.kmin[d] = lo[d];
        h.kext[d] = hi[d] - lo[d] + 1;
      }
    }
    h.nfw = c.nfw;
    h.ns = c.ns;
    h.ntype = c.ntype;
    h.nk = c.nk;
    for (int i = 0; i < gm.natoms; ++i) {
      h.qs[i] = gm.chg[i];
      h.chgea[i] = gm.chg[i] / s.epsq * fmc::kR4pie0;  // ewald.f:688 (chgea)
      h.qsf[i] = (float)h.qs[i];
      h.chgeaf[i] = (float)h.chgea[i];
    }
    a->volm = s.volm;
    a->rcut = s.rcut;
    a->engunit = s.engunit;
    a->dlrpot = s.dlrpot;
    for (int i = 0; i < gm.natoms; ++i)
      for (int k = 0; k < c.ntype; ++k)
        if (gm.ltp[i] == a->type_of_field[k])
          raise(FMC_ERR_INPUT, "the adjoint needs guest and framework atom types apart");
    a->eps0.assign((size_t)c.ns * c.ntype, 0.0);
    a->sig0.assign((size_t)c.ns * c.ntype, 0.0);
    for (int i = 0; i < c.ns; ++i)
      for (int k = 0; k < c.ntype; ++k) {
        const int iv = s.lstvdw[fmc::loc2(gm.ltp[i], a->type_of_field[k])];
        if (iv < 1 || iv > s.ntpvdw || s.ltpvdw[iv] != 2)
          raise(FMC_ERR_INPUT, "the adjoint needs a 12-6 LJ pair for every guest site and framework type");
        a->eps0[(size_t)i * c.ntype + k] = s.prmvdw[iv][1];
        a->sig0[(size_t)i * c.ntype + k] = s.prmvdw[iv][2];
      }
    a->ntyp.assign(c.ntype, 0.0);
    for (int j = 0; j < c.nfw; ++j) a->ntyp[fwt[j]] += 1.0;
    const size_t ts = (size_t)h.tabstride;
    std::vector<double> erc(ts, 0.0);
    for (int i = 1; i <= s.mxegrd; ++i) erc[i] = s.erc[i];
    a->erc64.upload(erc);
    a->erc32.upload(std::vector<float>(erc.begin(), erc.end()));
    std::vector<double> vgg;
    for (int i = 0; i < c.ns; ++i)
      for (int j = 0; j < c.ns; ++j) {
        const int iv = s.lstvdw[fmc::loc2(gm.ltp[i], gm.ltp[j])];
        h.gg_row[i][j] = -1;
        if (iv >= 1 && iv <= s.ntpvdw) {
          h.gg_row[i][j] = (int)(vgg.size() / ts);
          for (size_t q = 0; q < ts; ++q) vgg.push_back(q >= 1 && (int)q <= s.mxegrd ? s.vvv[iv][q] : 0.0);
        }
      }
    if (vgg.empty()) vgg.assign(ts, 0.0);
    a->vgg64.upload(vgg);
    a->vgg32.upload(std::vector<float>(vgg.begin(), vgg.end()));
    {  // framework atoms wrapped into the cell and sorted by (type, cell), cells z fastest
      const int T = c.ntype;
      std::vector<double4> wf(c.nfw);
      std::vector<int> key(c.nfw), order(c.nfw);
      for (int j = 0; j < c.nfw; ++j) {
        double p3[3] = {fw[j].x, fw[j].y, fw[j].z};
        int ic[3];
        for (int d = 0; d < 3; ++d) {
          p3[d] -= h.L[d] * std::floor(p3[d] * h.rL[d]);
          ic[d] = std::min(h.nc[d] - 1, (int)(p3[d] * h.rL[d] * h.nc[d]));
        }
        wf[j] = make_double4(p3[0], p3[1], p3[2], fw[j].w);
        key[j] = fwt[j] * (h.nc[0] * h.nc[1] * h.nc[2]) + (ic[0] * h.nc[1] + ic[1]) * h.nc[2] + ic[2];
        order[j] = j;
      }
      std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return key[x] < key[y]; });
      const int nkey = h.nc[0] * h.nc[1] * h.nc[2] * T;
      std::vector<int> cs(nkey + 1, 0);
      for (int j = 0; j < c.nfw; ++j) cs[key[j] + 1]++;
      for (int q = 0; q < nkey; ++q) cs[q + 1] += cs[q];
      std::vector<double4> sf(c.nfw);
      std::vector<float4> hi(c.nfw), lo(c.nfw);
      for (int j = 0; j < c.nfw; ++j) {
        const double4 a = wf[order[j]];
        sf[j] = a;
        const float hx = (float)a.x, hy = (float)a.y, hz = (float)a.z;
        hi[j] = make_float4(hx, hy, hz, (float)a.w);
        lo[j] = make_float4((float)(a.x - hx), (float)(a.y - hy), (float)(a.z - hz), 0.f);
      }
      a->hfw.upload(sf);
      a->hfwh.upload(hi);
      a->hfwl.upload(lo);
      a->hcstart.upload(cs);
    }
    {
      std::vector<double4> kv(std::max(1, c.nk));
      for (int k = 0; k < c.nk; ++k)
        kv[k] = make_double4(2.0 * fmc::kPi * s.kl[k] * c.rL[0], 2.0 * fmc::kPi * s.km[k] * c.rL[1],
                             2.0 * fmc::kPi * s.kn[k] * c.rL[2], -2.0 * c.krecip * s.akk[k]);
      a->kv.upload(kv);
      std::vector<float4> kv32(kv.size()), klf(kv.size());
      for (size_t k = 0; k < kv.size(); ++k) {
        kv32[k] = make_float4((float)kv[k].x, (float)kv[k].y, (float)kv[k].z, (float)kv[k].w);
        klf[k] = k < (size_t)c.nk ? make_float4((float)s.kl[k], (float)s.km[k], (float)s.kn[k], 0.f)
                                  : make_float4(0.f, 0.f, 0.f, 0.f);
      }
      a->kv32.upload(kv32);
      a->klf.upload(klf);
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

int fmc_adjoint_eval_batch(fmc_adjoint *a, int nsnap, const int *nmol, const double *xyz,
                           const double *params, int precision, double *energy, float *gxyz,
                           double *gparams) {
  return aguard([&] {
    if (!a || (nsnap > 0 && (!nmol || !params || !energy || !gparams))) raise(FMC_ERR_ARG, "null argument");
    if (nsnap < 0) raise(FMC_ERR_ARG, "negative snapshot count");
    if (precision != FMC_PREC_FP32 && precision != FMC_PREC_FP64) raise(FMC_ERR_ARG, "bad precision");
    HamConst h = a->h;
    const int T = h.ntype, ns = h.ns;
    for (int t = 0; t < T; ++t) {
      if (!(params[3 * t] >= 0.0) || !(params[3 * t + 1] > 0.0))
        raise(FMC_ERR_ARG, "epsilon >= 0 and sigma > 0 required");
      h.eps_t[t] = params[3 * t];
      h.lam[t] = params[3 * t + 2];
      h.lamf[t] = (float)h.lam[t];
    }
    std::vector<int> mol_snap, mol0(std::max(1, nsnap)), nm(std::max(1, nsnap));
    long long total = 0;
    for (int q = 0; q < nsnap; ++q) {
      if (nmol[q] < 0) raise(FMC_ERR_ARG, "negative molecule count");
      mol0[q] = (int)total;
      nm[q] = nmol[q];
      total += nmol[q];
      if (total * ns > (1LL << 26)) raise(FMC_ERR_CAPACITY, "too many guest sites in one batch");
      for (int i = 0; i < nmol[q]; ++i) mol_snap.push_back(q);
    }
    if (total > 0 && (!xyz || !gxyz)) raise(FMC_ERR_ARG, "null argument");
    // the guest-framework tables at these parameters (forgen's expression,
    // vdw_terms.f:181-234, with Lorentz-Berthelot moves of the FIELD's pair
    // values) and their sigma derivatives
    const size_t ts = (size_t)h.tabstride;
    std::vector<double> vt((size_t)ns * T * ts, 0.0), ds((size_t)ns * T * ts, 0.0);
    std::vector<double> pe((size_t)ns * T), ps((size_t)ns * T);
    for (int i = 0; i < ns; ++i)
      for (int t = 0; t < T; ++t) {
        const size_t o = (size_t)i * T + t;
        const double e0t = a->c.par[t][0], s0t = a->c.par[t][1];
        const double eps = a->eps0[o] * (e0t > 0.0 ? std::sqrt(params[3 * t] / e0t) : 0.0);
        const double sig = a->sig0[o] + 0.5 * (params[3 * t + 1] - s0t);
        pe[o] = eps;
        ps[o] = sig;
        for (int q = 1; q <= h.mxegrd; ++q) {
          const double rr = double(q) * a->dlrpot;
          const double sr6 = std::pow(sig / rr, 6);
          vt[o * ts + q] = 4.0 * eps * sr6 * (sr6 - 1.0);
          ds[o * ts + q] = 0.5 * 4.0 * eps * (12.0 * sr6 * sr6 - 6.0 * sr6) / sig;
        }
      }
    auto &W = a->w;
    auto &dms = W.dms, &dm0 = W.dm0, &dnm = W.dnm;
    auto &e_d = W.e_d, &p_d = W.p_d, &g64 = W.g64, &vt64 = W.vt64, &ds64 = W.ds64;
    auto &vt32 = W.vt32, &ds32 = W.ds32;
    auto &fr = W.fr, &cw = W.cw, &sgf = W.sgf;
    auto &sg = W.sg;
    dms.put(mol_snap.empty() ? std::vector<int>{0} : mol_snap);
    dm0.put(mol0);
    dnm.put(nm);
    e_d.reserve(std::max(1, nsnap));
    p_d.reserve((size_t)std::max(1, nsnap) * 3 * T);
    FMC_ACUDA(cudaMemset(e_d.p, 0, e_d.n * sizeof(double)));
    FMC_ACUDA(cudaMemset(p_d.p, 0, p_d.n * sizeof(double)));
    g64.reserve((size_t)std::max(1LL, total) * ns * 3);
    if (precision == FMC_PREC_FP64) {
      vt64.put(vt);
      ds64.put(ds);
    } else {
      vt32.put(std::vector<float>(vt.begin(), vt.end()));
      ds32.put(std::vector<float>(ds.begin(), ds.end()));
    }
    fr.reserve((size_t)std::max(1LL, total) * ns * 3);
    cw.reserve((size_t)std::max(1LL, total) * ns * 3);
    sg.reserve((size_t)std::max(1, nsnap) * std::max(1, h.nk));
    if (precision == FMC_PREC_FP32) sgf.reserve((size_t)std::max(1, nsnap) * std::max(1, h.nk));
    if (total > 0) {
      const int nsite = (int)(total * ns);
      ham_frac_kernel<<<(3 * nsite + 255) / 256, 256>>>(h, xyz, nsite, fr.p, cw.p);
      FMC_ACUDA(cudaGetLastError());
      if (precision == FMC_PREC_FP64) {
        ham_real_kernel<double><<<(unsigned)total, kHT>>>(
            h, a->hfw.p, a->hfwh.p, a->hfwl.p, a->hcstart.p, xyz, cw.p, dms.p, dm0.p, dnm.p, a->erc64.p,
            vt64.p, ds64.p, a->vgg64.p, g64.p, e_d.p, p_d.p);
      } else {
        ham_real_kernel<float><<<(unsigned)total, kHT>>>(
            h, a->hfw.p, a->hfwh.p, a->hfwl.p, a->hcstart.p, xyz, cw.p, dms.p, dm0.p, dnm.p, a->erc32.p,
            vt32.p, ds32.p, a->vgg32.p, g64.p, e_d.p, p_d.p);
      }
      FMC_ACUDA(cudaGetLastError());
      if (h.nk > 0) {
        dim3 grid(nsnap, (h.nk + kHT - 1) / kHT);  // snapshots along x (up to 2^31 - 1)
        if (precision == FMC_PREC_FP64)
          ham_sk_kernel<double><<<grid, kHT>>>(h, a->klmn.p, a->akk.p, a->skt.p, xyz, fr.p, dm0.p, dnm.p,
                                               sg.p, e_d.p, p_d.p);
        else {
          FMC_ACUDA(cudaFuncSetAttribute(ham_sk32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)ham_sk32_smem(h)));
          ham_sk32_kernel<<<grid, kHT, ham_sk32_smem(h)>>>(h, a->klmn.p, a->akk.p, a->skt.p, fr.p, dm0.p,
                                                           dnm.p, sg.p, sgf.p, e_d.p, p_d.p);
        }
        FMC_ACUDA(cudaGetLastError());
      }
      const unsigned gb = (unsigned)((total + 127) / 128);
      if (precision == FMC_PREC_FP64)
        ham_recip_grad_kernel<double><<<gb, 128>>>(h, a->klmn.p, a->kv.p, sg.p, xyz, fr.p, dms.p,
                                                  (int)total, g64.p, gxyz);
      else if (ns == 3)  // three-site guests (CO2) with their site loops unrolled
        ham_recip_grad32_kernel<3><<<gb, 128>>>(h, a->klmn.p, a->klf.p, a->kv32.p, sgf.p, fr.p, dms.p,
                                                (int)total, g64.p, gxyz);
      else
        ham_recip_grad32_kernel<kMaxASite><<<gb, 128>>>(h, a->klmn.p, a->klf.p, a->kv32.p, sgf.p, fr.p,
                                                        dms.p, (int)total, g64.p, gxyz);
      FMC_ACUDA(cudaGetLastError());
    }
    FMC_ACUDA(cudaDeviceSynchronize());
    std::vector<double> e(std::max(1, nsnap)), gp((size_t)std::max(1, nsnap) * 3 * T);
    FMC_ACUDA(cudaMemcpy(e.data(), e_d.p, e.size() * sizeof(double), cudaMemcpyDeviceToHost));
    FMC_ACUDA(cudaMemcpy(gp.data(), p_d.p, gp.size() * sizeof(double), cudaMemcpyDeviceToHost));
    // the guest-framework Lennard-Jones tail (lrcorrect, vdw_terms.f:470-645):
    // 2 pi / V n_a n_t eadd per site and framework type, eadd = 2 x 4 eps
    // (sigma^12 / (9 rc^9) - sigma^6 / (3 rc^3)) for unlike types
    const double rc = a->rcut, twopi = 2.0 * fmc::kPi;
    for (int q = 0; q < nsnap; ++q) {
      const double N = double(nmol[q]);
      for (int i = 0; i < ns; ++i)
        for (int t = 0; t < T; ++t) {
          const size_t o = (size_t)i * T + t;
          const double eps = pe[o], sig = ps[o];
          const double pre = twopi / a->volm * N * a->ntyp[t] / a->engunit;
          const double eadd = 2.0 * 4.0 * eps * (std::pow(sig, 12) / (9.0 * std::pow(rc, 9)) -
                                                 std::pow(sig, 6) / (3.0 * std::pow(rc, 3)));
          const double dsig = 2.0 * 4.0 * eps * (12.0 * std::pow(sig, 11) / (9.0 * std::pow(rc, 9)) -
                                                 6.0 * std::pow(sig, 5) / (3.0 * std::pow(rc, 3)));
          e[q] += pre * eadd;
          if (params[3 * t] > 0.0) gp[(size_t)q * 3 * T + 3 * t] += pre * eadd / (2.0 * params[3 * t]);
          gp[(size_t)q * 3 * T + 3 * t + 1] += pre * dsig * 0.5;
        }
      energy[q] = e[q];
      for (int j = 0; j < 3 * T; ++j) gparams[(size_t)q * 3 * T + j] = gp[(size_t)q * 3 * T + j];
    }
    return FMC_OK;
  });
}

int fmc_adjoint_destroy(fmc_adjoint *a) {
  delete a;
  return FMC_OK;
}

}  // extern "C"

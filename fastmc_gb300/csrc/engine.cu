// engine.cu -- kernels and the C ABI of the GB300 GCMC energy path.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "engine.cuh"
#include "fmc_internal.h"

using namespace fmcdev;

namespace fmc {

thread_local std::string g_error;
void set_error(const std::string &m) { g_error = m; }
[[noreturn]] void raise(int code, const std::string &msg) { throw Error{code, msg}; }

#define FMC_CUDA(x)                                                                \
  do {                                                                             \
    cudaError_t e_ = (x);                                                          \
    if (e_ != cudaSuccess)                                                         \
      ::fmc::raise(FMC_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <class F>
int guard(F &&f) {
  try {
    g_error.clear();
    return f();
  } catch (const Error &e) {
    g_error = e.msg;
    return e.code;
  } catch (const std::exception &e) {
    g_error = e.what();
    return FMC_ERR_ARG;
  }
}

// --------------------------------------------------------------- kernels
// K4: full structure factor S(k) = sum_j q_j e^{i k.r_j} of a set of atoms
// (ewald.f:354-661).  Each block handles kKB k-vectors; threads stride
// over the atoms; FP64 throughout.
constexpr int kKB = 8;
struct Rcell {
  double r[9];
};

__global__ void __launch_bounds__(kThreads) structure_factor_kernel(
    const double4 *__restrict__ atoms, int n, const int4 *__restrict__ klmn, int nk, Rcell rc,
    double2 *__restrict__ out) {
  __shared__ double red[kWarps * 2 * kKB + 2 * kKB];
  int k0 = blockIdx.x * kKB;
  double ax[kKB], ay[kKB];
  int4 kv[kKB];
  for (int j = 0; j < kKB; ++j) {
    ax[j] = ay[j] = 0.0;
    kv[j] = (k0 + j < nk) ? klmn[k0 + j] : make_int4(0, 0, 0, 0);
  }
  for (int a = threadIdx.x; a < n; a += kThreads) {
    double4 A = atoms[a];
    double f[3];
    for (int d = 0; d < 3; ++d) f[d] = rc.r[d] * A.x + rc.r[3 + d] * A.y + rc.r[6 + d] * A.z;
    for (int j = 0; j < kKB; ++j) {
      double t = double(kv[j].x) * f[0] + double(kv[j].y) * f[1] + double(kv[j].z) * f[2];
      t -= rint(t);
      double sn, cs;
      sincospi(2.0 * t, &sn, &cs);
      ax[j] += A.w * cs;
      ay[j] += A.w * sn;
    }
  }
  double vals[2 * kKB];
  for (int j = 0; j < kKB; ++j) {
    vals[2 * j] = ax[j];
    vals[2 * j + 1] = ay[j];
  }
  block_sum(vals, 2 * kKB, red);
  if (threadIdx.x < kKB && k0 + threadIdx.x < nk) {
    const double *R = red + kWarps * 2 * kKB;
    out[k0 + threadIdx.x] = make_double2(R[2 * threadIdx.x], R[2 * threadIdx.x + 1]);
  }
}

// FP32 issue-rate probe: 16 independent FMA chains per thread, so that the
// FMA pipes, not their latency, bound it (2 flops per FMA).
constexpr int kProbeChains = 16;
__global__ void __launch_bounds__(256) fma_probe_kernel(float *out, int iters, float b, float c) {
  float a[kProbeChains];
#pragma unroll
  for (int j = 0; j < kProbeChains; ++j) a[j] = (float)(threadIdx.x + j) * 1e-6f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < kProbeChains; ++j) a[j] = fmaf(a[j], b, c);
  }
  float t = 0.f;
#pragma unroll
  for (int j = 0; j < kProbeChains; ++j) t += a[j];
  if (t == 12345.678f) out[0] = t;  // keeps the loop; practically never stores
}

// The chain kernel's instantiations (chain_f32_g1.cu, chain_f32_g4.cu,
// chain_f64.cu): launch wrappers, shared-memory set-up, cluster occupancy.
template <bool F32, int GN>
cudaError_t launch_chain(int nchains, int csize, const int *chain_ids, size_t smem,
                         cudaStream_t stream, const SysDev *systems, ChainHdr *hdrs,
                         const ChainArrays &CA, MoveCtx *gctx, LogRec *logs, int logcap,
                         int nmoves, int mode, const double *ctl_fuga, const WidomJob &wj);
template <bool F32, int GN>
cudaError_t set_chain_smem(size_t smem);
template <bool F32, int GN>
cudaError_t max_clusters(int csize, size_t smem, int *out);
#define FMC_CHAIN_EXTERN(F32, GN)                                                               \
  extern template cudaError_t launch_chain<F32, GN>(int, int, const int *, size_t, cudaStream_t, \
                                                    const SysDev *, ChainHdr *,                  \
                                                    const ChainArrays &, MoveCtx *, LogRec *, int, \
                                                    int, int, const double *, const WidomJob &); \
  extern template cudaError_t set_chain_smem<F32, GN>(size_t);                                   \
  extern template cudaError_t max_clusters<F32, GN>(int, size_t, int *);
FMC_CHAIN_EXTERN(true, 1)
FMC_CHAIN_EXTERN(true, kMaxG)
FMC_CHAIN_EXTERN(false, kMaxG)
#undef FMC_CHAIN_EXTERN

// Modes of the chain kernel (chain_kernel.cuh).
constexpr int kModeMoves = 0;
constexpr int kModeCreate = 1;
constexpr int kModeEval = 2;
constexpr int kModeCommit = 3;
constexpr int kModeWidom = 4;
constexpr int kModeLoad = 5;

// ----------------------------------------------------- device allocations
// Every cudaMalloc / cudaFree the library makes goes through DBuf and is
// counted here (fmc_alloc_count).
std::atomic<long long> g_dev_allocs{0}, g_dev_frees{0};

template <class T>
struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  ~DBuf() { release(); }
  void release() {
    if (p) {
      cudaFree(p);
      g_dev_frees.fetch_add(1);
    }
    p = nullptr;
  }
  void alloc(size_t count) {
    release();
    n = count;
    if (count) {
      FMC_CUDA(cudaMalloc(&p, count * sizeof(T)));
      g_dev_allocs.fetch_add(1);
    }
  }
  void upload(const std::vector<T> &v) {
    alloc(v.size());
    if (!v.empty()) FMC_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  }
  void zero() {
    if (p) FMC_CUDA(cudaMemset(p, 0, n * sizeof(T)));
  }
};

// Device copy of one system (framework, tables, k-vectors, S_fw).
struct DevSystem {
  SysDev d{};
  DBuf<double4> fw64;
  DBuf<float4> fwhi, fwlo, cpad_hi, cpad_lo;
  DBuf<int> fwtype, cell_start, pairtab, numtyp_fw, numfrz_fw;
  DBuf<double> erc, vvv, sig2, steadd, akk;
  DBuf<float4> ercq, vvvq;
  DBuf<float> akk32, sig2f;
  DBuf<float4> skfw_df;
  DBuf<int4> klmn;
  DBuf<unsigned> kpk;
  DBuf<double2> skfw;
  std::vector<double2> skfw_host;
  const System *host = nullptr;
};

void ensure_device() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) raise(FMC_ERR_NODEVICE, "no CUDA device is visible");
}

std::vector<float4> quad_coeffs(const std::vector<double> &tab, int mx) {
  std::vector<float4> q(mx + 3, make_float4(0, 0, 0, 0));
  for (int l = 1; l <= mx; ++l) {
    double v0 = tab[l], v1 = tab[l + 1], v2 = (l + 2 < (int)tab.size()) ? tab[l + 2] : 0.0;
    double D = v2 - 2.0 * v1 + v0;
    const float a = (float)v0;
    q[l] = make_float4(a, (float)(v1 - v0 - 0.5 * D), (float)(0.5 * D), (float)(v0 - (double)a));
  }
  return q;
}

void compute_sk(const std::vector<double4> &atoms, const DevSystem &D, double2 *out) {
  DBuf<double4> a;
  a.upload(atoms);
  Rcell rc;
  for (int i = 0; i < 9; ++i) rc.r[i] = D.d.rcell[i];
  int nb = (D.d.nk + kKB - 1) / kKB;
  if (nb > 0) structure_factor_kernel<<<nb, kThreads>>>(a.p, (int)atoms.size(), D.klmn.p, D.d.nk, rc, out);
  FMC_CUDA(cudaGetLastError());
  FMC_CUDA(cudaDeviceSynchronize());
}

void build_device_system(const System &s, DevSystem &D) {
  ensure_device();
  D.host = &s;
  SysDev &d = D.d;
  std::memset(&d, 0, sizeof d);
  d.imcon = s.imcon;
  for (int i = 0; i < 9; ++i) {
    d.cell[i] = s.cell[i];
    d.rcell[i] = s.rcell[i];
    d.cellh[i] = (float)s.cell[i];
    d.celll[i] = (float)(s.cell[i] - (double)d.cellh[i]);
    d.rcellh[i] = (float)s.rcell[i];
    d.rcelll[i] = (float)(s.rcell[i] - (double)d.rcellh[i]);
  }
  d.box[0] = s.cell[0];
  d.box[1] = s.cell[4];
  d.box[2] = s.cell[8];
  for (int dd = 0; dd < 3; ++dd) {
    d.rbox[dd] = 1.0 / d.box[dd];
    d.boxh[dd] = (float)d.box[dd];
    d.boxl[dd] = (float)(d.box[dd] - (double)d.boxh[dd]);
    d.rboxf[dd] = (float)d.rbox[dd];
    d.rboxf_lo[dd] = (float)(d.rbox[dd] - (double)d.rboxf[dd]);
  }
  d.volm = s.volm;
  d.statvolm = s.statvolm;
  d.temp = s.temp;
  d.beta = s.beta;
  d.engunit = s.engunit;
  d.rengunit = 1.0 / s.engunit;
  d.epsq = s.epsq;
  d.alpha = s.alpha;
  d.rcut = s.rcut;
  d.rc2 = s.rcut * s.rcut;
  d.overlap_sq = s.overlap_sq;
  d.overlap_sqf = (float)s.overlap_sq;
  d.rc2f = (float)(s.rcut * s.rcut);
  d.surftol = s.surftol;
  d.sumchg0 = s.sumchg;
  d.maxmls = s.maxmls;
  d.ntpguest = s.ntpguest;
  d.ntpatm = s.ntpatm;
  d.fw_mol = s.fw_mol;
  d.eqsteps = s.eqsteps;
  d.nwindsteps = s.nwindsteps;
  d.minchk = s.minchk;
  d.laccsample = s.laccsample ? 1 : 0;
  if (s.ntpatm > kMaxT) raise(FMC_ERR_INPUT, "too many atom types");
  for (int dd = 0; dd < 3; ++dd) {
    d.kmax[dd] = s.kmax[dd];
    if (s.kmax[dd] + 1 > kMaxKm) raise(FMC_ERR_INPUT, "kmax beyond the supported 39");
  }
  // framework atoms: sort into cells (z fastest) for imcon 1/2
  const MolType &fw = s.mol[s.fw_mol];
  int n = fw.nummols * fw.natoms;
  d.nfw = n;
  std::vector<double> x(n), y(n), z(n), q(n);
  std::vector<int> t(n);
  double chg_fw = 0.0;
  for (int i = 0; i < n; ++i) {
    x[i] = fw.xyz[3 * i];
    y[i] = fw.xyz[3 * i + 1];
    z[i] = fw.xyz[3 * i + 2];
    q[i] = fw.chg[i % fw.natoms];
    t[i] = fw.ltp[i % fw.natoms];
    chg_fw += q[i];
  }
  d.chgsum_fw = chg_fw;
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::vector<int> cstart;
  d.use_cells = (s.imcon == 1 || s.imcon == 2) ? 1 : 0;
  if (d.use_cells) {
    for (int dd = 0; dd < 3; ++dd) {
      d.nc[dd] = std::max(3, (int)std::floor(d.box[dd] / 2.5));
      d.csz[dd] = d.box[dd] / d.nc[dd];
      d.rcsz[dd] = 1.0 / d.csz[dd];
      d.rcszf[dd] = (float)d.rcsz[dd];
      d.cszf[dd] = (float)d.csz[dd];
    }
    std::vector<int> cell(n);
    for (int i = 0; i < n; ++i) {
      double w[3] = {x[i], y[i], z[i]};
      int c3[3];
      for (int dd = 0; dd < 3; ++dd) {
        w[dd] -= d.box[dd] * std::floor(w[dd] / d.box[dd]);
        c3[dd] = std::min(d.nc[dd] - 1, std::max(0, (int)std::floor(w[dd] / d.csz[dd])));
      }
      x[i] = w[0];
      y[i] = w[1];
      z[i] = w[2];
      cell[i] = (c3[0] * d.nc[1] + c3[1]) * d.nc[2] + c3[2];
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cell[a] < cell[b]; });
    int ncell = d.nc[0] * d.nc[1] * d.nc[2];
    cstart.assign(ncell + 1, 0);
    for (int i = 0; i < n; ++i) cstart[cell[i] + 1]++;
    for (int c = 0; c < ncell; ++c) cstart[c + 1] += cstart[c];
  } else {
    cstart = {0, n};
  }
  std::vector<double4> a64(n);
  std::vector<float4> ahi(n), alo(n);
  std::vector<int> at(n);
  for (int i = 0; i < n; ++i) {
    int o = order[i];
    a64[i] = make_double4(x[o], y[o], z[o], q[o]);
    float hx = (float)x[o], hy = (float)y[o], hz = (float)z[o];
    ahi[i] = make_float4(hx, hy, hz, (float)q[o]);
    alo[i] = make_float4((float)(x[o] - hx), (float)(y[o] - hy), (float)(z[o] - hz),
                         (float)(q[o] - (double)(float)q[o]));
    at[i] = t[o];
  }
  D.fw64.upload(a64);
  D.fwhi.upload(ahi);
  D.fwlo.upload(alo);
  D.fwtype.upload(at);
  D.cell_start.upload(cstart);
  if (d.use_cells) {
    int ncell = d.nc[0] * d.nc[1] * d.nc[2], maxc = 1;
    for (int c = 0; c < ncell; ++c) maxc = std::max(maxc, cstart[c + 1] - cstart[c]);
    int lp = 0;
    while ((1 << lp) < maxc) ++lp;
    const int pad = 1 << lp;
    std::vector<float4> ph((size_t)ncell * pad, make_float4(1e18f, 1e18f, 1e18f, 0.f));
    std::vector<float4> pl((size_t)ncell * pad, make_float4(0.f, 0.f, 0.f, 0.f));
    for (int c = 0; c < ncell; ++c)
      for (int j = 0; j < cstart[c + 1] - cstart[c]; ++j) {
        ph[(size_t)c * pad + j] = ahi[cstart[c] + j];
        pl[(size_t)c * pad + j] = alo[cstart[c] + j];
      }
    D.cpad_hi.upload(ph);
    D.cpad_lo.upload(pl);
    d.cpad_log2 = lp;
    d.cpad_hi = D.cpad_hi.p;
    d.cpad_lo = D.cpad_lo.p;
  }
  d.fw64 = D.fw64.p;
  d.fwhi = D.fwhi.p;
  d.fwlo = D.fwlo.p;
  d.fwtype = D.fwtype.p;
  d.cell_start = D.cell_start.p;
  // tables
  d.mxegrd = s.mxegrd;
  d.tabstride = s.mxegrd + 3;
  d.rdrewd = 1.0 / s.drewd;
  d.rdlrpot = 1.0 / s.dlrpot;
  d.rdrewdf = (float)d.rdrewd;
  d.rdlrpotf = (float)d.rdlrpot;
  d.rdlrpotf_lo = (float)(d.rdlrpot - (double)d.rdlrpotf);
  std::vector<double> erc(d.tabstride, 0.0);
  for (int i = 1; i <= s.mxegrd; ++i) erc[i] = s.erc[i];
  D.erc.upload(erc);
  D.ercq.upload(quad_coeffs(erc, s.mxegrd));
  int ntab = s.ntpvdw + 1;
  std::vector<double> vvv((size_t)ntab * d.tabstride, 0.0);
  std::vector<float4> vq((size_t)ntab * d.tabstride, make_float4(0, 0, 0, 0));
  for (int k = 1; k <= ntab && k < (int)s.vvv.size(); ++k) {
    std::vector<double> row(d.tabstride, 0.0);
    for (int i = 1; i <= s.mxegrd; ++i) row[i] = s.vvv[k][i];
    std::copy(row.begin(), row.end(), vvv.begin() + (size_t)(k - 1) * d.tabstride);
    auto qq = quad_coeffs(row, s.mxegrd);
    std::copy(qq.begin(), qq.end(), vq.begin() + (size_t)(k - 1) * d.tabstride);
  }
  D.vvv.upload(vvv);
  D.vvvq.upload(vq);
  int na = s.ntpatm + 1;
  std::vector<int> ptab(na * na, -1);
  std::vector<double> sig2(na * na, 0.0);
  for (int a = 1; a <= s.ntpatm; ++a)
    for (int b = 1; b <= s.ntpatm; ++b) {
      int k = s.lstvdw[loc2(a, b)];
      if (k >= 1 && k <= ntab && s.ltpvdw[k] < 100 && std::fabs(s.vvv[k][1]) > 1.0e-10)
        ptab[a * na + b] = k - 1;
      double sg = (k >= 1 && k < (int)s.prmvdw.size()) ? s.prmvdw[k][2] : 0.0;
      double st = s.surftol + sg;
      sig2[a * na + b] = st * st;
    }
  D.pairtab.upload(ptab);
  D.sig2.upload(sig2);
  std::vector<float> sig2f(sig2.begin(), sig2.end());
  D.sig2f.upload(sig2f);
  d.sig2f = D.sig2f.p;
  D.steadd.upload(s.steadd);
  D.numtyp_fw.upload(s.numtyp_fw);
  D.numfrz_fw.upload(s.numfrz_fw);
  d.erc = D.erc.p;
  d.vvv = D.vvv.p;
  d.ercq = D.ercq.p;
  d.vvvq = D.vvvq.p;
  d.pairtab = D.pairtab.p;
  d.sig2 = D.sig2.p;
  d.steadd = D.steadd.p;
  d.numtyp_fw = D.numtyp_fw.p;
  d.numfrz_fw = D.numfrz_fw.p;
  // k vectors
  d.nk = s.newld;
  // FP32 path arrays are padded to whole tiles of kKT k-vectors: padding
  // entries are k = (0,0,0) with a_k = 0 and S_fw = 0, so they add nothing
  const int nkpad = std::max(1, (s.newld + kKT - 1) / kKT) * kKT;
  std::vector<int4> lmn(s.newld);
  std::vector<float> a32(nkpad, 0.0f);
  for (int dd = 0; dd < 3; ++dd)
    if (s.kmax[dd] + 1 > kMaxKm)
      raise(FMC_ERR_INPUT, "kmax above " + std::to_string(kMaxKm - 1) + " is not supported");
  // packed k for the FP32 loop: l * (2 kmax_y + 1) + m + kmax_y | (n + 128) << 16
  const int wlm = 2 * s.kmax[1] + 1;
  std::vector<unsigned> pk(nkpad, (unsigned)s.kmax[1] | (128u << 16));
  for (int k = 0; k < s.newld; ++k) {
    lmn[k] = make_int4(s.kl[k], s.km[k], s.kn[k], 0);
    a32[k] = (float)s.akk[k];
    if (s.kl[k] < 0 || s.kl[k] > s.kmax[0] || std::abs(s.km[k]) > s.kmax[1] ||
        std::abs(s.kn[k]) > s.kmax[2])
      raise(FMC_ERR_INPUT, "k-vector index outside kmax");
    pk[k] = (unsigned)(s.kl[k] * wlm + s.km[k] + s.kmax[1]) | ((unsigned)(s.kn[k] + 128) << 16);
  }
  D.klmn.upload(lmn);
  D.kpk.upload(pk);
  D.akk.upload(s.akk);
  D.akk32.upload(a32);
  d.kpk = D.kpk.p;
  d.klmn = D.klmn.p;
  d.akk = D.akk.p;
  d.akk32 = D.akk32.p;
  d.krecip = 2.0 * (2.0 * kPi / s.volm) * kR4pie0 / s.epsq;
  // probability grids: (subgrid, site) items per guest type, in storeprob's
  // order (utility_pack.f:636-685)
  d.prob_nsub = s.lprob ? s.ntprob : 0;
  for (int k = 0; k < 3; ++k) d.ngrid[k] = s.ngrid[k];
  d.prob_gridsize = s.lprob ? s.ngrid[0] * s.ngrid[1] * s.ngrid[2] : 0;
  for (int k = 0; k < 9; ++k) d.rucell[k] = s.rucell[k];
  {
    int nit = 0, itprob = 0;
    for (int ig = 1; ig <= s.ntpguest; ++ig) {
      d.prob_item0[ig - 1] = nit;
      d.prob_nitem[ig - 1] = 0;
      d.prob_eng_sub[ig - 1] = -1;
      if (!s.lprob) continue;
      int np = s.nprob[ig];
      if (s.lprobeng[ig]) np -= 2;
      const int natms = s.mol[s.locguest[ig]].natoms;
      for (int ip = 1; ip <= np; ++ip) {
        const int sub = itprob + ip;
        if (sub > s.ntprob) raise(FMC_ERR_INPUT, "probability blocks inconsistent");
        for (int j = 1; j <= s.nprobsites[sub]; ++j) {
          const int site = s.lprobsites[sub][j];
          if (site < 0 || site > natms) raise(FMC_ERR_INPUT, "probability site index out of range");
          if (nit >= kMaxProbItems) raise(FMC_ERR_CAPACITY, "too many probability-grid sites");
          d.prob_sub[nit] = (short)(sub - 1);
          d.prob_site[nit] = (short)site;
          ++nit;
          d.prob_nitem[ig - 1]++;
        }
      }
      itprob += np;
      if (s.lprobeng[ig]) {  // the guest type's last two grids (storeenprob)
        itprob += 2;
        d.prob_eng_sub[ig - 1] = itprob - 2;
      }
    }
  }
  // framework S(k) (K4)
  D.skfw.alloc(std::max(1, s.newld));
  compute_sk(a64, D, D.skfw.p);
  D.skfw_host.resize(s.newld);
  if (s.newld)
    FMC_CUDA(cudaMemcpy(D.skfw_host.data(), D.skfw.p, s.newld * sizeof(double2), cudaMemcpyDeviceToHost));
  d.skfw = D.skfw.p;
  {
    std::vector<float4> df(nkpad, make_float4(0.f, 0.f, 0.f, 0.f));
    for (int k = 0; k < s.newld; ++k) {
      double2 v = D.skfw_host[k];
      float hx = (float)v.x, hy = (float)v.y;
      df[k] = make_float4(hx, hy, (float)(v.x - (double)hx), (float)(v.y - (double)hy));
    }
    D.skfw_df.upload(df);
    d.skfw_df = D.skfw_df.p;
  }
  // guest types
  for (int g = 1; g <= s.ntpguest; ++g) {
    GuestType &G = d.g[g - 1];
    const MolType &m = s.mol[s.locguest[g]];
    G.mol = s.locguest[g];
    G.ns = m.natoms;
    G.rns = 1.0f / (float)m.natoms;
    G.insert0 = s.guest_insert[g];
    double cx = 0, cy = 0, cz = 0;
    for (int i = 0; i < m.natoms; ++i) {
      G.q[i] = m.chg[i];
      G.mass[i] = m.wght[i];
      G.type[i] = m.ltp[i];
      G.frz[i] = m.frz[i];
      for (int dd = 0; dd < 3; ++dd) G.tmpl[i][dd] = s.guest_tmpl[g][3 * i + dd];
      cx += G.tmpl[i][0];
      cy += G.tmpl[i][1];
      cz += G.tmpl[i][2];
    }
    cx /= m.natoms;
    cy /= m.natoms;
    cz /= m.natoms;
    double rmax = 0.0;
    for (int i = 0; i < m.natoms; ++i) {
      double dx = G.tmpl[i][0] - cx, dy = G.tmpl[i][1] - cy, dz = G.tmpl[i][2] - cz;
      rmax = std::max(rmax, std::sqrt(dx * dx + dy * dy + dz * dz));
    }
    G.rmax = rmax;
    for (int i = 0; i < kMaxS; ++i)
      for (int t = 0; t <= kMaxT; ++t) {
        G.prow[i][t] = -1;
        G.psig2[i][t] = 0.f;
      }
    for (int i = 0; i < m.natoms; ++i)
      for (int t = 0; t <= s.ntpatm && t <= kMaxT; ++t) {
        const int pi = m.ltp[i] * (s.ntpatm + 1) + t;
        G.prow[i][t] = ptab[pi];
        G.psig2[i][t] = (float)sig2[pi];
      }
    {
      double mt = 0.0;
      for (int i = 0; i < m.natoms; ++i) mt += m.wght[i];
      for (int i = 0; i < m.natoms; ++i) {
        for (int dd = 0; dd < 3; ++dd) {
          G.tmplf[i][dd] = (float)G.tmpl[i][dd];
          G.tmplf_lo[i][dd] = (float)(G.tmpl[i][dd] - (double)G.tmplf[i][dd]);
        }
        G.wf[i] = (float)(m.wght[i] / mt);
        G.wf_lo[i] = (float)(m.wght[i] / mt - (double)G.wf[i]);
      }
    }
    G.ewald3en = s.ewald3en[G.mol];
    double qs = 0.0, q2 = 0.0, mass = 0.0;
    for (int i = 0; i < m.natoms; ++i) {
      qs += m.chg[i];
      q2 += m.chg[i] * m.chg[i];
      mass += m.wght[i];
    }
    double r4 = kR4pie0 / s.epsq;
    for (int i = 0; i < m.natoms; ++i) {
      G.chgea[i] = m.chg[i] / s.epsq * kR4pie0;  // ewald.f:688 (chgea)
      G.chgeaf[i] = (float)G.chgea[i];
      G.chgeaf_lo[i] = (float)(G.chgea[i] - (double)G.chgeaf[i]);
    }
    G.chgtmp = qs;
    G.engsic0 = -r4 * s.alpha * q2 / kSqrPi;  // ewald.f:105
    G.qfa = -(0.5 * kPi * r4) * (qs / s.alpha) / s.volm;  // ewald.f:317-318
    G.qfb = -(0.5 * kPi * r4) * ((qs / s.alpha) * (qs / s.alpha)) / s.volm;
    G.qfm = -(kPi * r4) * qs / (s.alpha * s.alpha * s.volm);  // ewald.f:336-337
    G.rmass = 1.0 / mass;
    // gstlrcorrect (vdw_terms.f:686-776) as a linear function of the
    // guest counts: per unique type pair k = 2 pi / V * eadd(i,j).
    {
      std::vector<int> ntg(s.ntpatm + 1, 0), nfg(s.ntpatm + 1, 0);
      for (int i = 0; i < m.natoms; ++i) {
        ntg[m.ltp[i]]++;
        if (m.frz[i]) nfg[m.ltp[i]]++;
      }
      double A = 0.0, Cc = 0.0, Bv[kMaxG] = {0, 0, 0, 0};
      int iv = 0;
      for (int i = 1; i <= s.ntpatm; ++i)
        for (int j = 1; j <= i; ++j) {
          ++iv;
          double kk = 2.0 * kPi / s.volm * s.steadd[iv];
          double na = ntg[i], nb = ntg[j], fa = nfg[i], fb = nfg[j];
          double pfw = na * s.numtyp_fw[j] + nb * s.numtyp_fw[i] - fa * s.numfrz_fw[j] -
                       fb * s.numfrz_fw[i];
          double self = na * nb - fa * fb;
          A += kk * (pfw + self);
          Cc += kk * self;
          for (int g2 = 1; g2 <= s.ntpguest; ++g2) {
            const MolType &m2 = s.mol[s.locguest[g2]];
            double t2i = 0, t2j = 0, f2i = 0, f2j = 0;
            for (int q = 0; q < m2.natoms; ++q) {
              if (m2.ltp[q] == i) {
                t2i += 1;
                if (m2.frz[q]) f2i += 1;
              }
              if (m2.ltp[q] == j) {
                t2j += 1;
                if (m2.frz[q]) f2j += 1;
              }
            }
            Bv[g2 - 1] += kk * (na * t2j + nb * t2i - fa * f2j - fb * f2i);
          }
        }
      G.lrcA = A;
      G.lrcC = Cc;
      for (int g2 = 0; g2 < kMaxG; ++g2) G.lrcB[g2] = Bv[g2];
    }
    G.delr = s.delr[g];
    G.disp_ratio = s.disp_ratio[g];
    G.tran_ratio = s.tran_ratio[g];
    G.rota_ratio = s.rota_ratio[g];
    G.mcinsf = s.mcinsf[g];
    G.mcdelf = s.mcdelf[g];
    G.mcdisf = s.mcdisf[g];
    G.mcjmpf = s.mcjmpf[g];
    G.mcswpf = s.mcswpf[g];
    G.mctraf = s.mctraf[g];
    G.mcrotf = s.mcrotf[g];
    G.mcswif = s.mcswif[g];
  }
}

// Initial chain header (alloc_config_arrays defaults, gcmc.f:389-399, 692-699).
ChainHdr initial_header(const System &s, int system_index, long long seed,
                        const double *fuga_override) {
  ChainHdr h;
  std::memset(&h, 0, sizeof h);
  long long sd = seed < 0 ? -seed : seed;
  int ms = int(sd % 1000), sec = int((sd / 1000) % 60);
  duni_init(h, ms, sec);
  h.system = system_index;
  for (int g = 1; g <= s.ntpguest; ++g) {
    h.delrdisp[g - 1] = s.delr[g];
    h.tran_delr[g - 1] = s.delr[g];
    h.fuga[g - 1] = s.gstfuga[g];
  }
  if (fuga_override && *fuga_override >= 0.0) h.fuga[0] = *fuga_override;
  h.rotangle = kPi / 3.0;
  h.rota_rotangle = h.rotangle;
  for (int g = 0; g < kMaxG; ++g) sync_step_pairs(h, g);
  h.production = s.eqsteps == 0 ? 1 : 0;
  h.minchk_left = std::max(1, s.minchk);
  h.window_left = std::max(1, s.nwindsteps);
  h.sumchg = s.sumchg;
  const MolType &fw = s.mol[s.fw_mol];
  double cf = 0.0;
  for (int i = 0; i < fw.natoms; ++i) cf += fw.chg[i] * fw.nummols;
  // chgsum_mol(framework) accumulates atom by atom in ewald1
  double acc = 0.0;
  for (int m = 0; m < fw.nummols; ++m)
    for (int i = 0; i < fw.natoms; ++i) acc += fw.chg[i];
  (void)cf;
  h.chgsum_mol[s.fw_mol] = acc;
  for (int a = 1; a <= s.ntpatm && a <= kMaxT; ++a) {
    h.numtyp[a] = s.numtyp_fw[a];
    h.numfrz[a] = s.numfrz_fw[a];
    h.numtyp_mol[s.fw_mol][a] = s.numtyp_fw[a];
    h.numfrz_mol[s.fw_mol][a] = s.numfrz_fw[a];
  }
  return h;
}

// A set of chains on the device (the per-move ABI uses one chain).
struct Chains {
  std::vector<std::unique_ptr<DevSystem>> sys;
  std::vector<const System *> hsys;
  DBuf<SysDev> sysarr;
  DBuf<ChainHdr> hdr;
  DBuf<double> gpos;
  DBuf<float4> ghi, glo;
  DBuf<int> ord, freel;
  DBuf<double2> sk, snew, sold, sksave;
  DBuf<float4> skdf, skdf2;
  DBuf<float4> trig;  // sin/cos(2 pi k / kTrigN) hi/lo pairs
  DBuf<double> grid;  // probability grids [chain][subgrid][bin]
  DBuf<MoveCtx> ctx;
  DBuf<LogRec> logs;
  DBuf<double> ctl_fuga;
  ChainArrays CA{};
  int nchains = 0, precision = 0, logcap = 0, maxmls = 0;
  int device = -1;  // the CUDA device the chains were created on
  int gn = kMaxG;  // guest-type capacity of the kernel's accumulators (1 or kMaxG)
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaGraphExec_t graph = nullptr;
  int graph_moves = -1;
  size_t smem = 0;
  bool headers_stale = true;  // host_hdr no longer mirrors the device headers
  double last_ms = 0.0;
  long long last_evals = 0, last_moves = 0;
  std::vector<ChainHdr> host_hdr;
  // chains grouped by the cluster size of their system; one launch per
  // group, the groups on their own streams (parallel branches of the graph)
  struct Group {
    int csize = 1, n = 0;
    DBuf<int> ids;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
  };
  std::vector<int> csys;    // cluster size per system (the last per-system setting)
  std::vector<int> cchain;  // cluster size per chain
  std::vector<std::unique_ptr<Group>> groups;
  cudaEvent_t fork = nullptr;

  ~Chains() {
    for (auto &g : groups) {
      if (g->done) cudaEventDestroy(g->done);
      if (g->stream) cudaStreamDestroy(g->stream);
    }
    if (fork) cudaEventDestroy(fork);
    if (graph) cudaGraphExecDestroy(graph);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
  }

  cudaError_t launch_one(int n, int csize, const int *ids, cudaStream_t st, int mode, int nmoves,
                         const WidomJob &wj = WidomJob{}) {
    if (precision == FMC_PREC_FP32 && gn == 1)
      return launch_chain<true, 1>(n, csize, ids, smem, st, sysarr.p, hdr.p, CA, ctx.p, logs.p,
                                   logcap, nmoves, mode, ctl_fuga.p, wj);
    if (precision == FMC_PREC_FP32)
      return launch_chain<true, kMaxG>(n, csize, ids, smem, st, sysarr.p, hdr.p, CA, ctx.p,
                                       logs.p, logcap, nmoves, mode, ctl_fuga.p, wj);
    return launch_chain<false, kMaxG>(n, csize, ids, smem, st, sysarr.p, hdr.p, CA, ctx.p, logs.p,
                                      logcap, nmoves, mode, ctl_fuga.p, wj);
  }

  int occupancy(int csize) {
    int n = 0;
    cudaError_t e;
    if (precision == FMC_PREC_FP32 && gn == 1) e = max_clusters<true, 1>(csize, smem, &n);
    else if (precision == FMC_PREC_FP32) e = max_clusters<true, kMaxG>(csize, smem, &n);
    else e = max_clusters<false, kMaxG>(csize, smem, &n);
    FMC_CUDA(e);
    return n;
  }

  // Per-system cluster sizes: every chain of system i on cs[i] CTAs.
  void set_clusters(const std::vector<int> &cs) {
    if (host_hdr.size() != (size_t)nchains || headers_stale) pull_headers();
    for (int v : cs)
      if (v < 1 || v > kMaxCluster) raise(FMC_ERR_ARG, "cluster size must be 1..8");
    std::vector<int> cc(nchains);
    for (int c = 0; c < nchains; ++c) cc[c] = cs[host_hdr[c].system];
    set_chain_clusters(cc);
    csys = cs;
  }

  // Regroup the chains after a change of their cluster sizes: one launch
  // (graph branch) per distinct size.
  // Size 0 pauses a chain: it is left out of the launches until it gets a
  // size again.
  void set_chain_clusters(const std::vector<int> &cc) {
    int active = 0;
    for (int v : cc) {
      if (v < 0 || v > kMaxCluster) raise(FMC_ERR_ARG, "cluster size must be 0..8");
      active += v > 0;
    }
    if (active == 0) raise(FMC_ERR_ARG, "every chain paused");
    for (auto &g : groups) {
      if (g->done) cudaEventDestroy(g->done);
      if (g->stream) cudaStreamDestroy(g->stream);
    }
    groups.clear();
    cchain = cc;
    csys.clear();
    for (int v = 1; v <= kMaxCluster; ++v) {
      std::vector<int> ids;
      for (int c = 0; c < nchains; ++c)
        if (cchain[c] == v) ids.push_back(c);
      if (ids.empty()) continue;
      if (v > 1 && occupancy(v) < 1)
        raise(FMC_ERR_ARG, "clusters of " + std::to_string(v) + " CTAs cannot be resident");
      auto g = std::make_unique<Group>();
      g->csize = v;
      g->n = (int)ids.size();
      g->ids.upload(ids);
      FMC_CUDA(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
      FMC_CUDA(cudaEventCreateWithFlags(&g->done, cudaEventDisableTiming));
      groups.push_back(std::move(g));
    }
    if (!fork) FMC_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    if (graph) {
      cudaGraphExecDestroy(graph);
      graph = nullptr;
    }
    graph_moves = -1;
  }

  void launch(int mode, int nmoves) {
    headers_stale = true;
    if (groups.empty() || (groups.size() == 1 && groups[0]->csize == 1 && groups[0]->n == nchains)) {
      FMC_CUDA(launch_one(nchains, 1, nullptr, stream, mode, nmoves));
      return;
    }
    // fork: every group waits for what is queued on the chain stream, and
    // the chain stream waits for every group
    FMC_CUDA(cudaEventRecord(fork, stream));
    for (auto &g : groups) {
      FMC_CUDA(cudaStreamWaitEvent(g->stream, fork, 0));
      FMC_CUDA(launch_one(g->n, g->csize, g->ids.p, g->stream, mode, nmoves));
      FMC_CUDA(cudaEventRecord(g->done, g->stream));
    }
    for (auto &g : groups) FMC_CUDA(cudaStreamWaitEvent(stream, g->done, 0));
  }

  void sync() { FMC_CUDA(cudaStreamSynchronize(stream)); }

  // FP32 path: every chain's guest S(k) back into skdf (the chain kernel
  // flips between skdf and skdf2 on accepted moves), before the host reads,
  // resets, snapshots or saves it.
  void normalize_sk() {
    if (precision != FMC_PREC_FP32 || !skdf2.p) return;
    pull_headers();
    bool any = false;
    for (int c = 0; c < nchains; ++c)
      for (int g = 0; g < kMaxG; ++g)
        if (host_hdr[c].skb[g]) {
          const size_t o = ((size_t)c * kMaxG + g) * CA.nkmax;
          FMC_CUDA(cudaMemcpyAsync(skdf.p + o, skdf2.p + o, CA.nkmax * sizeof(float4),
                                   cudaMemcpyDeviceToDevice, stream));
          host_hdr[c].skb[g] = 0;
          any = true;
        }
    if (any) {
      FMC_CUDA(cudaMemcpyAsync(hdr.p, host_hdr.data(), nchains * sizeof(ChainHdr),
                               cudaMemcpyHostToDevice, stream));
      sync();
    }
  }

  void pull_headers() {
    host_hdr.resize(nchains);
    FMC_CUDA(cudaMemcpyAsync(host_hdr.data(), hdr.p, nchains * sizeof(ChainHdr),
                             cudaMemcpyDeviceToHost, stream));
    sync();
    headers_stale = false;
  }

  void check_status() {
    pull_headers();
    for (int c = 0; c < nchains; ++c)
      if (host_hdr[c].status) {
        char buf[256];
        std::snprintf(buf, sizeof buf,
                      "chain %d raised device status 0x%x (1 table range, 2 segment overflow, "
                      "4 capacity, 8 non-finite, 16 bad molecule index, 32 kmax, "
                      "64 copy wait timed out, 128 generator buffer empty, "
                      "256 guest slot or position out of range)",
                      c, host_hdr[c].status);
        raise(FMC_ERR_DEVICE, buf);
      }
  }
};

void init_chains(Chains &C, const System *const *systems, int nsys, const fmc_chain_spec *spec,
                 int nchains, int precision, int cap) {
  ensure_device();
  if (nsys < 1 || nchains < 1) raise(FMC_ERR_ARG, "need at least one system and one chain");
  if (precision != FMC_PREC_FP64 && precision != FMC_PREC_FP32) raise(FMC_ERR_ARG, "bad precision");
  if (cap < 1 || cap > 4096) raise(FMC_ERR_ARG, "guest capacity must be in 1..4096");
  C.nchains = nchains;
  C.precision = precision;
  FMC_CUDA(cudaGetDevice(&C.device));
  int nkmax = 1, maxmls = 1;
  for (int i = 0; i < nsys; ++i) {
    if (!systems[i]) raise(FMC_ERR_ARG, "null system");
    auto D = std::make_unique<DevSystem>();
    build_device_system(*systems[i], *D);
    nkmax = std::max(nkmax, std::max(1, (systems[i]->newld + kKT - 1) / kKT) * kKT);
    maxmls = std::max(maxmls, systems[i]->maxmls);
    C.hsys.push_back(systems[i]);
    C.sys.push_back(std::move(D));
  }
  C.maxmls = maxmls;
  std::vector<SysDev> sd;
  for (auto &D : C.sys) sd.push_back(D->d);
  C.sysarr.upload(sd);
  std::vector<ChainHdr> hh;
  for (int c = 0; c < nchains; ++c) {
    int si = spec ? spec[c].system : 0;
    if (si < 0 || si >= nsys) raise(FMC_ERR_ARG, "chain system index out of range");
    double fu = spec ? spec[c].pressure_pa : -1.0;
    long long seed = spec ? (long long)spec[c].seed : 1;
    hh.push_back(initial_header(*systems[si], si, seed, &fu));
  }
  C.hdr.upload(hh);
  {
    std::vector<double> f(nchains);
    for (int c = 0; c < nchains; ++c) f[c] = hh[c].fuga[0];
    C.ctl_fuga.upload(f);
  }
  ChainArrays &CA = C.CA;
  CA.cap = cap;
  CA.nkmax = nkmax;
  size_t nsl = (size_t)nchains * kMaxG * cap * kMaxS;
  C.gpos.alloc(nsl * 3);
  C.gpos.zero();
  C.ghi.alloc(nsl);
  C.glo.alloc(nsl);
  C.ghi.zero();
  C.glo.zero();
  C.ord.alloc((size_t)nchains * kMaxG * cap);
  C.freel.alloc((size_t)nchains * kMaxG * cap);
  C.ord.zero();
  C.freel.zero();
  C.sk.alloc((size_t)nchains * kMaxG * nkmax);
  C.sk.zero();
  C.snew.alloc((size_t)nchains * nkmax);
  C.sold.alloc((size_t)nchains * nkmax);
  C.snew.zero();
  C.sold.zero();
  {  // the two guest types' S(k) for a rejection: FP64 chains with swap
    // moves, and chains whose switch moves can act (three or more guest
    // types; both precisions, FP32 entries are 16-byte hi/lo pairs too)
    bool swaps = false, switches = false;
    for (int i = 0; i < nsys; ++i)
      for (int g = 1; g <= systems[i]->ntpguest; ++g) {
        if (systems[i]->mcswpf[g] > systems[i]->mcjmpf[g]) swaps = true;
        if (systems[i]->mcswif[g] > systems[i]->mcrotf[g] && systems[i]->ntpguest >= 3) switches = true;
      }
    if ((swaps && precision == FMC_PREC_FP64) || switches) C.sksave.alloc((size_t)nchains * 2 * nkmax);
  }
  C.skdf.alloc((size_t)nchains * kMaxG * nkmax);
  C.skdf.zero();
  if (precision == FMC_PREC_FP32) {
    C.skdf2.alloc((size_t)nchains * kMaxG * nkmax);
    C.skdf2.zero();
  }
  C.ctx.alloc(nchains);
  C.ctx.zero();
  C.logs.alloc(1);
  {  // sin and cos of 2 pi k / kTrigN as float hi/lo pairs (double-float quaternions)
    std::vector<float4> t(kTrigN);
    for (int k = 0; k < kTrigN; ++k) {
      float a[2], b[2];
      split_pair(std::sin(2.0 * kPi * k / kTrigN), a);
      split_pair(std::cos(2.0 * kPi * k / kTrigN), b);
      t[k] = make_float4(a[0], a[1], b[0], b[1]);
    }
    C.trig.alloc(kTrigN);
    FMC_CUDA(cudaMemcpy(C.trig.p, t.data(), kTrigN * sizeof(float4), cudaMemcpyHostToDevice));
  }
  CA.trig = C.trig.p;
  {  // probability grids, when any system asks for them
    size_t stride = 0;
    for (int i = 0; i < nsys; ++i) {
      const System &s = *systems[i];
      if (s.lprob) stride = std::max(stride, (size_t)s.ntprob * s.ngrid[0] * s.ngrid[1] * s.ngrid[2]);
    }
    CA.grid_stride = stride;
    CA.grid = nullptr;
    if (stride) {
      C.grid.alloc(stride * nchains);
      C.grid.zero();
      CA.grid = C.grid.p;
    }
  }
  CA.gpos = C.gpos.p;
  CA.ghi = C.ghi.p;
  CA.glo = C.glo.p;
  CA.ord = C.ord.p;
  CA.freel = C.freel.p;
  CA.sk = C.sk.p;
  CA.skdf = C.skdf.p;
  CA.snew = C.snew.p;
  CA.sold = C.sold.p;
  CA.sksave = C.sksave.p;
  CA.skdf2 = C.skdf2.p;
  FMC_CUDA(cudaStreamCreateWithFlags(&C.stream, cudaStreamNonBlocking));
  FMC_CUDA(cudaEventCreate(&C.ev0));
  FMC_CUDA(cudaEventCreate(&C.ev1));
  C.smem = precision == FMC_PREC_FP32 ? sizeof(BlockShared<true>) : sizeof(BlockShared<false>);
  int ngmax = 1, nsmax = 1;
  for (int i = 0; i < nsys; ++i) {
    ngmax = std::max(ngmax, systems[i]->ntpguest);
    for (int g = 1; g <= systems[i]->ntpguest; ++g)
      nsmax = std::max(nsmax, systems[i]->mol[systems[i]->locguest[g]].natoms);
  }
  // parallelepiped cells run on the multi-type FP32 kernel (the single-type
  // one is built for orthorhombic cells only) with the global guest arrays
  bool tric = false;
  for (int i = 0; i < nsys; ++i) tric = tric || systems[i]->imcon == 3;
  C.gn = (precision == FMC_PREC_FP32 && ngmax == 1 && !tric) ? 1 : kMaxG;
  // guests resident in shared memory during a launch (FP32, one guest type,
  // capacity x sites within the shared array); the per-move ABI keeps them
  // in global memory (its launches are single moves)
  CA.resident =
      (precision == FMC_PREC_FP32 && ngmax == 1 && cap * nsmax <= kGuestSmem && !tric) ? 1 : 0;
  CA.spec_max = 0;  // speculative rounds off unless asked for (fmc_batch_set_speculation)
  cudaError_t e;
  if (precision == FMC_PREC_FP32 && C.gn == 1) e = set_chain_smem<true, 1>(C.smem);
  else if (precision == FMC_PREC_FP32) e = set_chain_smem<true, kMaxG>(C.smem);
  else e = set_chain_smem<false, kMaxG>(C.smem);
  FMC_CUDA(e);
}

void fill_stats(const Chains &C, fmc_chain_stats *out) {
  for (int c = 0; c < C.nchains; ++c) {
    const ChainHdr &h = C.host_hdr[c];
    fmc_chain_stats &o = out[c];
    std::memset(&o, 0, sizeof o);
    o.moves = h.moves;
    o.evals = h.evals;
    o.overlap_exits = h.overlap_exits;
    for (int i = 0; i < 8; ++i) {
      o.attempts[i] = h.attempts[i];
      o.accepts[i] = h.accepts[i];
    }
    const System &s = *C.hsys[h.system];
    o.nummols = h.nummols[0];
    o.status = h.status;
    o.energy = h.energy[s.locguest[1]];
    if (h.wsum > 0) {
      o.avg_n = h.wacc[0][0] / h.wsum;
      o.avg_e = h.wacc[0][1] / h.wsum;
      o.avg_en = h.wacc[0][2] / h.wsum;
      o.avg_n2 = h.wacc[0][3] / h.wsum;
      o.avg_e2 = h.wacc[0][4] / h.wsum;
      o.avg_nf = h.wacc[0][5] / h.wsum;
      o.qst = h.wacc[0][6] / h.wsum;
      o.cv = h.wacc[0][7] / h.wsum;
    }
    o.prodcount = h.prodcount;
    o.windows = h.windows;
    o.device_ns = h.dev_ns;
    for (int i = 0; i < 16; ++i) o.phase_cycles[i] = h.phase_cycles[i];
    // per guest type: <N> and the reference's "standard error" of it, the
    // weighted standard deviation of the window averages (gcmc.f:1218-1241)
    for (int g = 0; g < s.ntpguest && g < FMC_MAX_GUEST_TYPES; ++g) {
      if (h.wsum <= 0) continue;
      const double m = h.wacc[g][0] / h.wsum;
      o.guest_avg_n[g] = m;
      o.guest_se_n[g] = std::sqrt(std::max(0.0, h.wsq[g] / h.wsum - m * m));
    }
  }
}


// ------------------------------------ full Ewald sum without allocation
// fmc_full_ewald_noalloc recomputes what fmc_full_ewald does without any
// device allocation.  Its scratch -- one FP64 partial energy per block of
// kKB k-vectors, then the total -- is this fixed array in the module's
// static device memory, shared by every engine on a device.  Each call
// writes every word it later reads (partials first, then the total), so
// nothing in it has to start at zero; two calls running at the same time on
// one device would overwrite each other's partials, which is why the host
// side serialises its calls with g_noalloc_mu and waits for the kernels
// before it returns.
constexpr int kNoallocScratchDoubles = 8192;  // 64 KiB: up to 8191 blocks = 65528 k-vectors
static __device__ __align__(256) double g_ewald_scratch[kNoallocScratchDoubles];

struct GuestSites {
  int ntp;
  int n[kMaxG];             // molecules of each guest type
  int ns[kMaxG];            // sites per molecule
  double q[kMaxG][kMaxS];   // site charges
};

// Variant of structure_factor_kernel for the guests of chain 0: each block
// takes kKB k-vectors, sums every guest type's S(k) over that type's atoms in
// molecule order straight from the chain's coordinate storage (the same atom
// order and per-thread striding as the staged-copy path), writes it to the
// chain's running sums (sk in FP64, skdf as FP32 hi/lo pairs; the other
// pointer is null), and leaves sum_j akk |S_fw + sum_g S_g|^2 of its
// k-vectors in partial[block].
__global__ void __launch_bounds__(kThreads) guest_ewald_kernel(
    const double *__restrict__ gpos, const int *__restrict__ ord, int cap, GuestSites gs,
    const int4 *__restrict__ klmn, int nk, Rcell rc, const double *__restrict__ akk,
    const double2 *__restrict__ skfw, double2 *sk, float4 *skdf, int nkmax,
    double *__restrict__ partial) {
  __shared__ double red[kWarps * 2 * kKB + 2 * kKB];
  __shared__ double eterm[kKB];
  const int k0 = blockIdx.x * kKB;
  const int jt = threadIdx.x;
  int4 kv[kKB];
  for (int j = 0; j < kKB; ++j) kv[j] = (k0 + j < nk) ? klmn[k0 + j] : make_int4(0, 0, 0, 0);
  double2 tot = make_double2(0.0, 0.0);
  if (jt < kKB && k0 + jt < nk) tot = skfw[k0 + jt];
  for (int g = 0; g < gs.ntp; ++g) {
    double ax[kKB], ay[kKB];
    for (int j = 0; j < kKB; ++j) ax[j] = ay[j] = 0.0;
    const int ns = gs.ns[g], na = gs.n[g] * ns;
    for (int a = threadIdx.x; a < na; a += kThreads) {
      const int i = a / ns, sidx = a - i * ns;
      const int slot = ord[(size_t)g * cap + i];
      const double *p = gpos + (((size_t)g * cap + slot) * kMaxS + sidx) * 3;
      const double x = p[0], y = p[1], z = p[2], q = gs.q[g][sidx];
      double f[3];
      for (int d = 0; d < 3; ++d) f[d] = rc.r[d] * x + rc.r[3 + d] * y + rc.r[6 + d] * z;
      for (int j = 0; j < kKB; ++j) {
        double t = double(kv[j].x) * f[0] + double(kv[j].y) * f[1] + double(kv[j].z) * f[2];
        t -= rint(t);
        double sn, cs;
        sincospi(2.0 * t, &sn, &cs);
        ax[j] += q * cs;
        ay[j] += q * sn;
      }
    }
    double vals[2 * kKB];
    for (int j = 0; j < kKB; ++j) {
      vals[2 * j] = ax[j];
      vals[2 * j + 1] = ay[j];
    }
    block_sum(vals, 2 * kKB, red);
    if (jt < kKB && k0 + jt < nk) {
      const double *R = red + kWarps * 2 * kKB;
      const double sx = R[2 * jt], sy = R[2 * jt + 1];
      const size_t o = (size_t)g * nkmax + k0 + jt;
      if (sk) sk[o] = make_double2(sx, sy);
      if (skdf) {
        const float hx = (float)sx, hy = (float)sy;
        skdf[o] = make_float4(hx, hy, (float)(sx - hx), (float)(sy - hy));
      }
      tot.x += sx;
      tot.y += sy;
    }
  }
  if (jt < kKB) eterm[jt] = (k0 + jt < nk) ? akk[k0 + jt] * (tot.x * tot.x + tot.y * tot.y) : 0.0;
  __syncthreads();
  if (threadIdx.x == 0) {
    double e = 0.0;
    for (int j = 0; j < kKB; ++j) e += eterm[j];
    partial[blockIdx.x] = e;
  }
}

// Sum of n partials into *out (one block).
__global__ void __launch_bounds__(kThreads) partial_sum_kernel(const double *__restrict__ partial,
                                                               int n, double *out) {
  __shared__ double red[kWarps + 1];
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += kThreads) v += partial[i];
  block_sum(&v, 1, red);
  if (threadIdx.x == 0) *out = red[kWarps];
}

std::mutex g_noalloc_mu;
constexpr int kNoallocDevices = 64;
double *g_noalloc_addr[kNoallocDevices] = {};

// Device address of g_ewald_scratch on the current device, looked up once
// per device (the first call on a device is the one that may load the
// module there).  Called with g_noalloc_mu held.
double *noalloc_scratch() {
  int dev = -1;
  FMC_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoallocDevices) raise(FMC_ERR_ARG, "device ordinal out of range");
  if (!g_noalloc_addr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_ewald_scratch);
    if (e != cudaSuccess || !p)
      raise(FMC_ERR_CUDA, std::string("cudaGetSymbolAddress of the static Ewald scratch: ") +
                              cudaGetErrorString(e));
    g_noalloc_addr[dev] = static_cast<double *>(p);
  }
  return g_noalloc_addr[dev];
}

}  // namespace fmc

// =================================================================== C ABI
using namespace fmc;

struct ChainSnapshot;

struct fmc_plain {
  Chains C;
  fmc_system_info info{};
  int has_move = 0;
  std::unique_ptr<ChainSnapshot> swap_saved;  // set while a swap awaits fmc_swap_finish
  // pinned host copies of the move record (one copy each way per evaluation)
  MoveCtx *pin_in = nullptr, *pin_out = nullptr;
  MoveCtx last{};                // the last evaluated move, for the host's decision
  int nummols[kMaxG] = {};       // host mirror of the guest counts (energy_eval's N)
  int swap_nummols[kMaxG] = {};  // the mirror before a pending swap
  ~fmc_plain() {
    if (pin_in) cudaFreeHost(pin_in);
    if (pin_out) cudaFreeHost(pin_out);
  }
};

// The per-move ABI runs its commit kernels asynchronously; everything that
// reads the engine's device state on another stream or on the host waits
// for them first.
static void settle(const fmc_plain *h) {
  FMC_CUDA(cudaStreamSynchronize(h->C.stream));
}

struct fmc_batch {
  Chains C;
  std::unique_ptr<ChainSnapshot> snap;  // fmc_batch_snapshot
};

// Device copy of every chain's mutable state (for trial runs).
struct ChainSnapshot {
  DBuf<ChainHdr> hdr;
  DBuf<double> gpos;
  DBuf<float4> ghi, glo, skdf;
  DBuf<int> ord, freel;
  DBuf<double2> sk;
  DBuf<double> grid;
};

template <class T>
static void copy_buf(DBuf<T> &dst, const DBuf<T> &src, cudaStream_t st) {
  if (dst.n != src.n) dst.alloc(src.n);
  if (src.n) FMC_CUDA(cudaMemcpyAsync(dst.p, src.p, src.n * sizeof(T), cudaMemcpyDeviceToDevice, st));
}

static void save_state(Chains &C, ChainSnapshot &s) {
  C.normalize_sk();
  copy_buf(s.hdr, C.hdr, C.stream);
  copy_buf(s.gpos, C.gpos, C.stream);
  copy_buf(s.ghi, C.ghi, C.stream);
  copy_buf(s.glo, C.glo, C.stream);
  copy_buf(s.skdf, C.skdf, C.stream);
  copy_buf(s.ord, C.ord, C.stream);
  copy_buf(s.freel, C.freel, C.stream);
  copy_buf(s.sk, C.sk, C.stream);
  copy_buf(s.grid, C.grid, C.stream);
  C.sync();
}

static void restore_state(Chains &C, ChainSnapshot &s) {
  copy_buf(C.hdr, s.hdr, C.stream);
  copy_buf(C.gpos, s.gpos, C.stream);
  copy_buf(C.ghi, s.ghi, C.stream);
  copy_buf(C.glo, s.glo, C.stream);
  copy_buf(C.skdf, s.skdf, C.stream);
  copy_buf(C.ord, s.ord, C.stream);
  copy_buf(C.freel, s.freel, C.stream);
  copy_buf(C.sk, s.sk, C.stream);
  copy_buf(C.grid, s.grid, C.stream);
  C.sync();
  C.headers_stale = true;
}

// Checkpoint file: a header of sizes, then every chain's mutable device
// arrays as raw bytes (state records, coordinates, order lists, S(k)).
static const char kCkptMagic[8] = {'F', 'M', 'C', 'G', 'B', '3', '0', '2'};

template <class T>
static void ckpt_write(std::FILE *f, const DBuf<T> &d) {
  std::vector<T> h(d.n);
  if (d.n) FMC_CUDA(cudaMemcpy(h.data(), d.p, d.n * sizeof(T), cudaMemcpyDeviceToHost));
  const unsigned long long n = d.n;
  if (std::fwrite(&n, sizeof n, 1, f) != 1 || (n && std::fwrite(h.data(), sizeof(T), n, f) != n))
    raise(FMC_ERR_ARG, "checkpoint write failed");
}

// One array of the checkpoint into host memory; its length must match the
// batch's device array.
template <class T>
static void ckpt_read(std::FILE *f, const DBuf<T> &d, std::vector<T> &h) {
  unsigned long long n = 0;
  if (std::fread(&n, sizeof n, 1, f) != 1 || n != d.n)
    raise(FMC_ERR_INPUT, "checkpoint does not match this batch (array size)");
  h.resize(n);
  if (n && std::fread(h.data(), sizeof(T), n, f) != n) raise(FMC_ERR_INPUT, "checkpoint truncated");
}

template <class T>
static void ckpt_upload(DBuf<T> &d, const std::vector<T> &h) {
  if (!h.empty()) FMC_CUDA(cudaMemcpy(d.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
}

// Every index a kernel takes from a chain record, order list or free list
// of a checkpoint is in range for this batch (the kernels trust them).
static void validate_headers(const Chains &C, const std::vector<ChainHdr> &hdr,
                             const std::vector<int> &ord, const std::vector<int> &freel) {
  const int cap = C.CA.cap;
  auto bad = [](int c, const char *what) {
    raise(FMC_ERR_INPUT, "checkpoint chain " + std::to_string(c) + ": " + what);
  };
  for (int c = 0; c < C.nchains; ++c) {
    const ChainHdr &h = hdr[c];
    if (h.system < 0 || h.system >= (int)C.sys.size()) bad(c, "refers to a missing system");
    const System &s = *C.hsys[h.system];
    if (h.ir < 1 || h.ir > 97 || h.jr < 1 || h.jr > 97) bad(c, "generator lags out of range");
    if (h.rhead < 0 || h.rhead >= kRBuf || h.ravail < 0 || h.ravail > kRBuf)
      bad(c, "generator buffer position out of range");
    if (h.log_n < 0) bad(c, "negative log position");
    for (int g = 0; g < kMaxG; ++g) {
      const int n = h.nummols[g], ns = h.nslots[g], nf = h.nfree[g];
      if (n < 0 || ns < 0 || nf < 0 || n > cap || ns > cap || nf > cap || n + nf > ns)
        bad(c, "guest counts out of range");
      if (g >= s.ntpguest && (n || ns || nf)) bad(c, "molecules of a guest type the system lacks");
      if (h.skb[g] != 0 && h.skb[g] != 1) bad(c, "structure-factor buffer flag not 0 or 1");
      const size_t base = ((size_t)c * kMaxG + g) * cap;
      for (int i = 0; i < n; ++i)
        if (ord[base + i] < 0 || ord[base + i] >= ns) bad(c, "molecule order entry out of range");
      for (int i = 0; i < nf; ++i)
        if (freel[base + i] < 0 || freel[base + i] >= ns) bad(c, "free-list entry out of range");
    }
  }
}

extern "C" {

int fmc_alloc_count(int64_t *allocs, int64_t *frees) {
  if (allocs) *allocs = g_dev_allocs.load();
  if (frees) *frees = g_dev_frees.load();
  return FMC_OK;
}

int fmc_measure_fp32_peak(double *tflops) {
  return guard([&] {
    if (!tflops) raise(FMC_ERR_ARG, "null argument");
    ensure_device();
    int dev = 0, nsm = 1;
    FMC_CUDA(cudaGetDevice(&dev));
    FMC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    DBuf<float> out;
    out.alloc(1);
    cudaEvent_t e0, e1;
    FMC_CUDA(cudaEventCreate(&e0));
    FMC_CUDA(cudaEventCreate(&e1));
    const int blocks = nsm * 8, threads = 256, iters = 1 << 14;
    double best = 0.0;
    for (int r = 0; r < 4; ++r) {  // the first launch warms the clocks up
      FMC_CUDA(cudaEventRecord(e0));
      fma_probe_kernel<<<blocks, threads>>>(out.p, iters, 0.999999f, 1e-7f);
      FMC_CUDA(cudaEventRecord(e1));
      FMC_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      FMC_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      const double flops = 2.0 * kProbeChains * (double)iters * blocks * threads;
      best = std::max(best, flops / (ms * 1e-3) / 1e12);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *tflops = best;
    return FMC_OK;
  });
}

int fmc_last_error(char *buf, int len) {
  int n = (int)g_error.size();
  if (buf && len > 0) {
    int m = std::min(n, len - 1);
    std::memcpy(buf, g_error.data(), m);
    buf[m] = 0;
  }
  return n;
}

const char *fmc_version(void) { return "fastmc_gb300 1.0 sm_103a"; }

int fmc_system_load(const char *dir, fmc_system **out) {
  return guard([&] {
    if (!out) raise(FMC_ERR_ARG, "null output pointer");
    auto p = std::make_unique<fmc_system>();
    load_system(dir ? dir : ".", p->s);
    *out = p.release();
    return FMC_OK;
  });
}

int fmc_upload_system(const fmc_system_desc *desc, fmc_system **out) {
  return guard([&] {
    if (!desc || !out) raise(FMC_ERR_ARG, "null argument");
    auto p = std::make_unique<fmc_system>();
    upload_system(*desc, p->s);
    *out = p.release();
    return FMC_OK;
  });
}

int fmc_system_free(fmc_system *sys) {
  delete sys;
  return FMC_OK;
}

int fmc_system_get_info(const fmc_system *sys, fmc_system_info *info) {
  return guard([&] {
    if (!sys || !info) raise(FMC_ERR_ARG, "null argument");
    const System &s = sys->s;
    std::memset(info, 0, sizeof *info);
    info->imcon = s.imcon;
    info->maxmls = s.maxmls;
    info->ntpguest = s.ntpguest;
    info->ntpatm = s.ntpatm;
    info->n_framework = s.mol[s.fw_mol].nummols * s.mol[s.fw_mol].natoms;
    for (int d = 0; d < 3; ++d) info->kmax[d] = s.kmax[d];
    info->newld = s.newld;
    info->mxegrd = s.mxegrd;
    for (int g = 1; g <= s.ntpguest; ++g) {
      info->guest_mol[g - 1] = s.locguest[g];
      info->guest_nsites[g - 1] = s.mol[s.locguest[g]].natoms;
      info->guest_insert[g - 1] = s.guest_insert[g];
      info->fugacity[g - 1] = s.gstfuga[g];
      info->ewald3en[g - 1] = s.ewald3en[s.locguest[g]];
    }
    info->alpha = s.alpha;
    info->rcut = s.rcut;
    info->volm = s.volm;
    info->engunit = s.engunit;
    info->temperature = s.temp;
    info->sumchg = s.sumchg;
    info->drewd = s.drewd;
    for (int i = 0; i < 9; ++i) info->cell[i] = s.cell[i];
    info->mcsteps = s.mcsteps;
    info->eqsteps = s.eqsteps;
    info->nwindsteps = s.nwindsteps;
    info->overlap = std::sqrt(s.overlap_sq);
    return FMC_OK;
  });
}

int fmc_system_set_fugacity(fmc_system *sys, int iguest, double pascal) {
  return guard([&] {
    if (!sys || iguest < 1 || iguest > sys->s.ntpguest) raise(FMC_ERR_ARG, "bad guest index");
    sys->s.gstfuga[iguest] = pascal;
    return FMC_OK;
  });
}

// ----------------------------------------------------------- plain mode
int fmc_plain_create(const fmc_system *sys, int precision, int guest_capacity, fmc_plain **out) {
  return guard([&] {
    if (!sys || !out) raise(FMC_ERR_ARG, "null argument");
    auto h = std::make_unique<fmc_plain>();
    const System *sp = &sys->s;
    fmc_chain_spec spec{0, -1.0, 1, 0};
    init_chains(h->C, &sp, 1, &spec, 1, precision, guest_capacity);
    h->C.CA.resident = 0;  // one move per launch: guests stay in global memory
    FMC_CUDA(cudaMallocHost(&h->pin_in, sizeof(MoveCtx)));
    FMC_CUDA(cudaMallocHost(&h->pin_out, sizeof(MoveCtx)));
    *out = h.release();
    return FMC_OK;
  });
}

int fmc_plain_destroy(fmc_plain *h) {
  delete h;
  return FMC_OK;
}

int fmc_full_ewald(fmc_plain *h, double *out4) {
  return guard([&] {
    if (!h || !out4) raise(FMC_ERR_ARG, "null argument");
    settle(h);
    Chains &C = h->C;
    C.normalize_sk();
    const System &s = *C.hsys[0];
    const DevSystem &D = *C.sys[0];
    C.pull_headers();
    const ChainHdr &hd = C.host_hdr[0];
    int nk = s.newld;
    // guest S(k) recomputed from the device coordinates, per guest type
    std::vector<double2> stot(D.skfw_host);
    double sq = 0.0, sumchg = 0.0;
    const MolType &fw = s.mol[s.fw_mol];
    for (int m = 0; m < fw.nummols; ++m)
      for (int i = 0; i < fw.natoms; ++i) {
        sq += fw.chg[i] * fw.chg[i];
        sumchg += fw.chg[i];
      }
    (void)sumchg;
    double e3 = 0.0;
    for (int g = 0; g < s.ntpguest; ++g) {
      int n = hd.nummols[g];
      const MolType &gm = s.mol[s.locguest[g + 1]];
      std::vector<int> ord(n);
      if (n)
        FMC_CUDA(cudaMemcpy(ord.data(), C.ord.p + (size_t)g * C.CA.cap, n * sizeof(int),
                            cudaMemcpyDeviceToHost));
      std::vector<double4> atoms;
      for (int i = 0; i < n; ++i) {
        std::vector<double> xyz(3 * kMaxS);
        FMC_CUDA(cudaMemcpy(xyz.data(), C.gpos.p + ((size_t)g * C.CA.cap + ord[i]) * kMaxS * 3,
                            3 * kMaxS * sizeof(double), cudaMemcpyDeviceToHost));
        for (int sidx = 0; sidx < gm.natoms; ++sidx) {
          atoms.push_back(make_double4(xyz[3 * sidx], xyz[3 * sidx + 1], xyz[3 * sidx + 2],
                                       gm.chg[sidx]));
          sq += gm.chg[sidx] * gm.chg[sidx];
        }
      }
      e3 += n * s.ewald3en[s.locguest[g + 1]];
      std::vector<double2> sg(nk, make_double2(0, 0));
      if (!atoms.empty() && nk) {
        DBuf<double2> tmp;
        tmp.alloc(nk);
        compute_sk(atoms, D, tmp.p);
        FMC_CUDA(cudaMemcpy(sg.data(), tmp.p, nk * sizeof(double2), cudaMemcpyDeviceToHost));
      }
      // reset the running S(k) of this guest type to the recomputed one
      if (nk && C.precision == FMC_PREC_FP32) {
        std::vector<float4> df(nk);
        for (int k = 0; k < nk; ++k) {
          float hx = (float)sg[k].x, hy = (float)sg[k].y;
          df[k] = make_float4(hx, hy, (float)(sg[k].x - hx), (float)(sg[k].y - hy));
        }
        FMC_CUDA(cudaMemcpy(C.skdf.p + (size_t)g * C.CA.nkmax, df.data(), nk * sizeof(float4),
                            cudaMemcpyHostToDevice));
      } else if (nk) {
        FMC_CUDA(cudaMemcpy(C.sk.p + (size_t)g * C.CA.nkmax, sg.data(), nk * sizeof(double2),
                            cudaMemcpyHostToDevice));
      }
      for (int k = 0; k < nk; ++k) {
        stot[k].x += sg[k].x;
        stot[k].y += sg[k].y;
      }
    }
    double eng = 0.0;
    for (int k = 0; k < nk; ++k) eng += s.akk[k] * (stot[k].x * stot[k].x + stot[k].y * stot[k].y);
    double r4 = fmc::kR4pie0 / s.epsq;
    double sic = -r4 * s.alpha * sq / fmc::kSqrPi;
    double qfix = -(0.5 * fmc::kPi * r4) * ((hd.sumchg / s.alpha) * (hd.sumchg / s.alpha) / s.volm);
    double ew1 = 2.0 * (2.0 * fmc::kPi / s.volm) * r4 * eng + sic + qfix;
    out4[0] = (ew1 - e3) / s.engunit;
    out4[1] = ew1;
    out4[2] = sic;
    out4[3] = qfix;
    return FMC_OK;
  });
}

static int plain_eval(fmc_plain *h, MoveCtx &mc, fmc_move_result *res, bool guest_energy) {
  Chains &C = h->C;
  if (h->swap_saved) raise(FMC_ERR_STATE, "a swap awaits fmc_swap_finish");
  const System &s = *C.hsys[0];
  mc.evaluated = 0;
  // the move up, one launch (after any commit still queued), the move back
  // with the chain's status word, one synchronisation
  *h->pin_in = mc;
  FMC_CUDA(cudaMemcpyAsync(C.ctx.p, h->pin_in, sizeof(MoveCtx), cudaMemcpyHostToDevice, C.stream));
  C.launch(kModeEval, 0);
  FMC_CUDA(cudaMemcpyAsync(h->pin_out, C.ctx.p, sizeof(MoveCtx), cudaMemcpyDeviceToHost, C.stream));
  C.sync();
  const MoveCtx &out = *h->pin_out;
  if (out.dev_status) {
    char buf[160];
    std::snprintf(buf, sizeof buf, "the chain raised device status 0x%x (see fmc_batch status bits)",
                  out.dev_status);
    raise(FMC_ERR_DEVICE, buf);
  }
  h->last = out;
  h->has_move = 1;
  if (res) {
    std::memset(res, 0, sizeof *res);
    res->estep = out.estep;
    if (guest_energy) res->estep = out.estep + out.delrc / s.engunit;
    res->ewld1 = out.parts[0];
    res->ewld2 = out.parts[1];
    res->vdw = out.parts[2];
    res->delrc = out.parts[3];
    for (int m = 1; m <= s.maxmls && m <= FMC_MAX_MOLTYPES; ++m) res->delE[m - 1] = out.delE[m];
    res->overlap = out.overlap;
    res->surface = out.surf_new;
    res->surface_old = out.surf_old;
    res->status = out.dev_status;
    for (int i = 0; i < out.ns && i < FMC_MAX_SITES; ++i)
      for (int d = 0; d < 3; ++d) res->newxyz[3 * i + d] = out.pos[0][i][d];
  }
  return FMC_OK;
}

int fmc_insertion(fmc_plain *h, int iguest, const double *xyz, fmc_move_result *res) {
  return guard([&] {
    if (!h || !xyz) raise(FMC_ERR_ARG, "null argument");
    const System &s = *h->C.hsys[0];
    if (iguest < 1 || iguest > s.ntpguest) raise(FMC_ERR_ARG, "bad guest index");
    MoveCtx mc;
    std::memset(&mc, 0, sizeof mc);
    mc.kind = 1;
    mc.g = iguest - 1;
    mc.ns = s.mol[s.locguest[iguest]].natoms;
    mc.npos = 1;
    mc.slot = -1;
    for (int i = 0; i < mc.ns; ++i)
      for (int d = 0; d < 3; ++d) mc.pos[0][i][d] = xyz[3 * i + d];
    return plain_eval(h, mc, res, false);
  });
}

int fmc_deletion(fmc_plain *h, int iguest, int choice, fmc_move_result *res) {
  return guard([&] {
    if (!h) raise(FMC_ERR_ARG, "null argument");
    const System &s = *h->C.hsys[0];
    if (iguest < 1 || iguest > s.ntpguest) raise(FMC_ERR_ARG, "bad guest index");
    MoveCtx mc;
    std::memset(&mc, 0, sizeof mc);
    mc.kind = 2;
    mc.g = iguest - 1;
    mc.ns = s.mol[s.locguest[iguest]].natoms;
    mc.npos = 1;
    mc.choice = choice;
    return plain_eval(h, mc, res, false);
  });
}

int fmc_guest_energy(fmc_plain *h, int iguest, int choice, fmc_move_result *res) {
  return guard([&] {
    if (!h) raise(FMC_ERR_ARG, "null argument");
    const System &s = *h->C.hsys[0];
    if (iguest < 1 || iguest > s.ntpguest) raise(FMC_ERR_ARG, "bad guest index");
    MoveCtx mc;
    std::memset(&mc, 0, sizeof mc);
    mc.kind = 2;
    mc.g = iguest - 1;
    mc.ns = s.mol[s.locguest[iguest]].natoms;
    mc.npos = 1;
    mc.choice = choice;
    int rc = plain_eval(h, mc, res, true);
    h->has_move = 0;  // an energy query is not a move to commit
    return rc;
  });
}

int fmc_displace(fmc_plain *h, int iguest, int choice, const double *abcq, fmc_move_result *res) {
  return guard([&] {
    if (!h || !abcq) raise(FMC_ERR_ARG, "null argument");
    const System &s = *h->C.hsys[0];
    if (iguest < 1 || iguest > s.ntpguest) raise(FMC_ERR_ARG, "bad guest index");
    MoveCtx mc;
    std::memset(&mc, 0, sizeof mc);
    mc.kind = 3;
    mc.g = iguest - 1;
    mc.ns = s.mol[s.locguest[iguest]].natoms;
    mc.npos = 2;
    mc.choice = choice;
    mc.pos[1][0][0] = abcq[0];
    mc.pos[1][0][1] = abcq[1];
    mc.pos[1][0][2] = abcq[2];
    mc.pos[1][1][0] = abcq[3];
    mc.pos[1][1][1] = abcq[4];
    mc.pos[1][1][2] = abcq[5];
    mc.pos[1][2][0] = abcq[6];
    return plain_eval(h, mc, res, false);
  });
}

// energy_eval (utility_pack.f:3637-3693) for the last evaluated move, on the
// host as the reference runs it, FP64: with N the guest count before the
// move, insert V f / ((N+1) kB T) e^{-beta dE}, delete N kB T / (V f)
// e^{-beta dE} (1 when f is zero), displace e^{-beta dE}, the exponent
// clamped at +-700; accepted when rande < test.  A displacement with
// estep < 0 is accepted without rande (gcmc.f:1879-1886); an overlapping
// insertion or displacement is rejected.
static int host_energy_eval(const fmc_plain *h, double rande) {
  const MoveCtx &m = h->last;
  const System &s = *h->C.hsys[0];
  if (m.kind == 0) return 0;
  if ((m.kind == 1 || m.kind >= 3) && m.overlap) return 0;
  if (m.kind >= 3 && m.estep < 0.0) return 1;
  const int g = m.g;
  const double eng = m.kind == 2 ? -m.estep : m.estep;
  const double ipress = s.gstfuga[g + 1];
  const int ing = h->nummols[g];
  double test = 0.0;
  if (-s.beta * eng > 700.0) test = std::exp(700.0);
  else if (s.beta * eng > 700.0) test = std::exp(-700.0);
  else if (m.kind >= 3) test = std::exp(-1.0 * s.beta * eng);
  else if (m.kind == 1)
    test = s.statvolm * ipress / ((double(ing) + 1.0) * fmc::kBoltz * s.temp) * std::exp(-1.0 * s.beta * eng);
  else if (std::fabs(ipress) < 1.0e-7) test = 1.0;
  else test = double(ing) * fmc::kBoltz * s.temp / (s.statvolm * ipress) * std::exp(-1.0 * s.beta * eng);
  return rande < test ? 1 : 0;
}

int fmc_metropolis_commit(fmc_plain *h, double rande, int *accepted) {
  return guard([&] {
    if (!h) raise(FMC_ERR_ARG, "null argument");
    if (!h->has_move) raise(FMC_ERR_STATE, "no evaluated move to commit");
    Chains &C = h->C;
    // decided here; accept_move (or nothing) queued on the engine's stream,
    // without waiting: the next evaluation runs after it
    const int acc = host_energy_eval(h, rande);
    C.launch(kModeCommit, acc);
    h->has_move = 0;
    if (acc && h->last.kind == 1) h->nummols[h->last.g]++;
    if (acc && h->last.kind == 2) h->nummols[h->last.g]--;
    if (accepted) *accepted = acc;
    return FMC_OK;
  });
}

int fmc_commit(fmc_plain *h, int accepted) {
  return guard([&] {
    if (!h) raise(FMC_ERR_ARG, "null argument");
    if (!h->has_move) raise(FMC_ERR_STATE, "no evaluated move to commit");
    const MoveCtx &m = h->last;
    // an overlapping insertion or displacement is never committed
    const int acc = (accepted && !((m.kind == 1 || m.kind >= 3) && m.overlap)) ? 1 : 0;
    h->C.launch(kModeCommit, acc);
    h->has_move = 0;
    if (acc && m.kind == 1) h->nummols[m.g]++;
    if (acc && m.kind == 2) h->nummols[m.g]--;
    return FMC_OK;
  });
}

static int chain_coords(const Chains &C, int chain, int iguest, double *xyz, int cap, int *nout);

// accept_move for the last evaluated move without energy_eval (mc_swap
// commits its deletion and its insertion before deciding)
static void forced_commit(fmc_plain *h) {
  Chains &C = h->C;
  MoveCtx mc;
  FMC_CUDA(cudaMemcpyAsync(&mc, C.ctx.p, sizeof(MoveCtx), cudaMemcpyDeviceToHost, C.stream));
  C.sync();
  mc.forced = 1;
  FMC_CUDA(cudaMemcpyAsync(C.ctx.p, &mc, sizeof(MoveCtx), cudaMemcpyHostToDevice, C.stream));
  C.launch(kModeCommit, -1);
  C.sync();
  C.check_status();
  if (!mc.overlap && mc.kind == 1) h->nummols[mc.g]++;
  if (mc.kind == 2) h->nummols[mc.g]--;
  h->has_move = 0;
}

int fmc_swap(fmc_plain *h, int iguest, int choice, int jguest, const double *q4,
             fmc_swap_result *res) {
  return guard([&] {
    if (!h || !q4) raise(FMC_ERR_ARG, "null argument");
    if (h->swap_saved) raise(FMC_ERR_STATE, "a swap awaits fmc_swap_finish");
    settle(h);
    Chains &C = h->C;
    const System &s = *C.hsys[0];
    std::memcpy(h->swap_nummols, h->nummols, sizeof h->nummols);
    if (iguest < 1 || iguest > s.ntpguest || jguest < 1 || jguest > s.ntpguest || jguest == iguest)
      raise(FMC_ERR_ARG, "bad guest index");
    const MolType &mi = s.mol[s.locguest[iguest]], &mj = s.mol[s.locguest[jguest]];
    const int ni = mi.natoms, nj = mj.natoms;
    ChainHdr hd;
    FMC_CUDA(cudaMemcpy(&hd, C.hdr.p, sizeof hd, cudaMemcpyDeviceToHost));
    const int nmols = hd.nummols[iguest - 1];
    if (choice < 1 || choice > nmols) raise(FMC_ERR_ARG, "bad molecule index");
    if (hd.nummols[jguest - 1] >= C.CA.cap) raise(FMC_ERR_CAPACITY, "guest capacity exceeded");
    // centre of mass of the chosen molecule (com, utility_pack.f)
    std::vector<double> xi((size_t)3 * ni * nmols);
    int nout = 0;
    chain_coords(C, 0, iguest, xi.data(), (int)xi.size(), &nout);
    const double *x = xi.data() + (size_t)3 * ni * (choice - 1);
    double c[3] = {0.0, 0.0, 0.0}, weight = 0.0;
    for (int i = 0; i < ni; ++i) {
      weight += mi.wght[i];
      for (int d = 0; d < 3; ++d) c[d] += x[3 * i + d] * mi.wght[i];
    }
    for (int d = 0; d < 3; ++d) c[d] /= weight;
    auto snap = std::make_unique<ChainSnapshot>();  // what a rejection restores
    save_state(C, *snap);
    // delete the first guest and commit it
    MoveCtx mc;
    std::memset(&mc, 0, sizeof mc);
    mc.kind = 2;
    mc.g = iguest - 1;
    mc.ns = ni;
    mc.npos = 1;
    mc.choice = choice;
    fmc_move_result r;
    plain_eval(h, mc, &r, false);
    const double estepi = -r.estep;
    forced_commit(h);
    // the partner type from its template at the centre of mass, rotated by
    // q about it (rotation, utility_pack.f:3480-3524)
    const double q1 = q4[0], q2 = q4[1], q3 = q4[2], qq = q4[3];
    const double Q[9] = {2.0 * q2 * q2 + 2.0 * q1 * q1 - 1.0, 2.0 * q2 * q3 - 2.0 * q1 * qq,
                         2.0 * q2 * qq + 2.0 * q1 * q3,       2.0 * q2 * q3 + 2.0 * q1 * qq,
                         2.0 * q1 * q1 + 2.0 * q3 * q3 - 1.0, 2.0 * q3 * qq - 2.0 * q1 * q2,
                         2.0 * q2 * qq - 2.0 * q1 * q3,       2.0 * q3 * qq + 2.0 * q1 * q2,
                         2.0 * qq * qq + 2.0 * q1 * q1 - 1.0};
    std::memset(&mc, 0, sizeof mc);
    mc.kind = 1;
    mc.g = jguest - 1;
    mc.ns = nj;
    mc.npos = 1;
    mc.slot = -1;
    const std::vector<double> &t = s.guest_tmpl[jguest];
    for (int i = 0; i < nj; ++i) {
      double v[3];
      for (int d = 0; d < 3; ++d) v[d] = (t[3 * i + d] + c[d]) - c[d];
      for (int d = 0; d < 3; ++d)
        mc.pos[0][i][d] = Q[3 * d] * v[0] + Q[3 * d + 1] * v[1] + Q[3 * d + 2] * v[2] + c[d];
    }
    fmc_move_result r2;
    plain_eval(h, mc, &r2, false);
    const double estepj = r2.estep;
    double testi = 0.0, testj = 0.0;
    if (!r2.overlap) {
      forced_commit(h);
      FMC_CUDA(cudaMemcpy(&hd, C.hdr.p, sizeof hd, cudaMemcpyDeviceToHost));
      // the reference's tests, its volume in cubic angstroms included
      const int jn = hd.nummols[jguest - 1], in = hd.nummols[iguest - 1] + 1;
      const double ipress = hd.fuga[iguest - 1], jpress = hd.fuga[jguest - 1];
      testi = double(in) * fmc::kBoltz * s.temp / (s.volm * ipress) * std::exp(-1.0 * s.beta * estepi);
      testj = s.volm * jpress / (double(jn) * fmc::kBoltz * s.temp) * std::exp(-1.0 * s.beta * estepj);
    }
    h->has_move = 0;
    h->swap_saved = std::move(snap);
    if (res) {
      std::memset(res, 0, sizeof *res);
      res->estepi = estepi;
      res->estepj = estepj;
      res->testi = testi;
      res->testj = testj;
      res->overlap = r2.overlap;
      for (int i = 0; i < 3 * nj && i < 3 * FMC_MAX_SITES; ++i) res->newxyz[i] = r2.newxyz[i];
    }
    return FMC_OK;
  });
}

int fmc_swap_finish(fmc_plain *h, int accepted) {
  return guard([&] {
    if (!h) raise(FMC_ERR_ARG, "null argument");
    if (!h->swap_saved) raise(FMC_ERR_STATE, "no swap to finish");
    if (!accepted) {
      restore_state(h->C, *h->swap_saved);
      std::memcpy(h->nummols, h->swap_nummols, sizeof h->nummols);
    }
    h->swap_saved.reset();
    return FMC_OK;
  });
}

int fmc_plain_get_nummols(const fmc_plain *h, int iguest, int *n) {
  return guard([&] {
    if (!h || !n) raise(FMC_ERR_ARG, "null argument");
    settle(h);
    ChainHdr hd;
    FMC_CUDA(cudaMemcpy(&hd, h->C.hdr.p, sizeof hd, cudaMemcpyDeviceToHost));
    if (iguest < 1 || iguest > kMaxG) raise(FMC_ERR_ARG, "bad guest index");
    *n = hd.nummols[iguest - 1];
    return FMC_OK;
  });
}

static int chain_coords(const Chains &C, int chain, int iguest, double *xyz, int cap, int *nout) {
  ChainHdr hd;
  FMC_CUDA(cudaMemcpy(&hd, C.hdr.p + chain, sizeof hd, cudaMemcpyDeviceToHost));
  const System &s = *C.hsys[hd.system];
  int g = iguest - 1;
  int n = hd.nummols[g];
  int ns = s.mol[s.locguest[iguest]].natoms;
  std::vector<int> ord(n);
  if (n)
    FMC_CUDA(cudaMemcpy(ord.data(), C.ord.p + ((size_t)chain * kMaxG + g) * C.CA.cap,
                        n * sizeof(int), cudaMemcpyDeviceToHost));
  std::vector<double> all((size_t)C.CA.cap * kMaxS * 3);
  FMC_CUDA(cudaMemcpy(all.data(), C.gpos.p + ((size_t)chain * kMaxG + g) * C.CA.cap * kMaxS * 3,
                      all.size() * sizeof(double), cudaMemcpyDeviceToHost));
  int w = 0;
  for (int i = 0; i < n; ++i)
    for (int sidx = 0; sidx < ns; ++sidx)
      for (int d = 0; d < 3; ++d) {
        if (w < cap) xyz[w] = all[((size_t)ord[i] * kMaxS + sidx) * 3 + d];
        ++w;
      }
  if (nout) *nout = n;
  return FMC_OK;
}

int fmc_plain_get_coords(const fmc_plain *h, int iguest, double *xyz, int cap) {
  return guard([&] {
    if (!h || !xyz) raise(FMC_ERR_ARG, "null argument");
    settle(h);
    return chain_coords(h->C, 0, iguest, xyz, cap, nullptr);
  });
}

static int chain_sk(Chains &C, int chain, double *out, int cap) {
  C.normalize_sk();
  ChainHdr hd;
  FMC_CUDA(cudaMemcpy(&hd, C.hdr.p + chain, sizeof hd, cudaMemcpyDeviceToHost));
  const System &s = *C.hsys[hd.system];
  const DevSystem &D = *C.sys[hd.system];
  int nk = s.newld, nm = s.maxmls + 1;
  if (cap < 2 * nm * nk) raise(FMC_ERR_CAPACITY, "output buffer too small for S(k)");
  std::vector<double2> g((size_t)kMaxG * C.CA.nkmax);
  if (C.precision == FMC_PREC_FP32) {
    std::vector<float4> df(g.size());
    FMC_CUDA(cudaMemcpy(df.data(), C.skdf.p + (size_t)chain * kMaxG * C.CA.nkmax,
                        df.size() * sizeof(float4), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < g.size(); ++i)
      g[i] = make_double2((double)df[i].x + (double)df[i].z, (double)df[i].y + (double)df[i].w);
  } else {
    FMC_CUDA(cudaMemcpy(g.data(), C.sk.p + (size_t)chain * kMaxG * C.CA.nkmax,
                        g.size() * sizeof(double2), cudaMemcpyDeviceToHost));
  }
  for (int k = 0; k < nk; ++k) {
    double tx = 0, ty = 0;
    for (int m = 0; m < nm; ++m) {
      out[2 * ((size_t)k * nm + m)] = 0.0;
      out[2 * ((size_t)k * nm + m) + 1] = 0.0;
    }
    double2 f = D.skfw_host[k];
    out[2 * ((size_t)k * nm + (s.fw_mol - 1))] = f.x;
    out[2 * ((size_t)k * nm + (s.fw_mol - 1)) + 1] = f.y;
    tx += f.x;
    ty += f.y;
    for (int gg = 0; gg < s.ntpguest; ++gg) {
      double2 v = g[(size_t)gg * C.CA.nkmax + k];
      int m = s.locguest[gg + 1] - 1;
      out[2 * ((size_t)k * nm + m)] = v.x;
      out[2 * ((size_t)k * nm + m) + 1] = v.y;
      tx += v.x;
      ty += v.y;
    }
    out[2 * ((size_t)k * nm + s.maxmls)] = tx;
    out[2 * ((size_t)k * nm + s.maxmls) + 1] = ty;
  }
  return FMC_OK;
}

int fmc_plain_get_sk(const fmc_plain *h, double *sk, int cap) {
  return guard([&] {
    if (!h || !sk) raise(FMC_ERR_ARG, "null argument");
    settle(h);
    // the buffer normalisation does not change what the handle holds
    return chain_sk(const_cast<fmc_plain *>(h)->C, 0, sk, cap);
  });
}

int fmc_plain_get_energy(const fmc_plain *h, double *energy, int cap) {
  return guard([&] {
    if (!h || !energy) raise(FMC_ERR_ARG, "null argument");
    settle(h);
    ChainHdr hd;
    FMC_CUDA(cudaMemcpy(&hd, h->C.hdr.p, sizeof hd, cudaMemcpyDeviceToHost));
    for (int m = 1; m <= h->C.maxmls && m <= cap; ++m) energy[m - 1] = hd.energy[m];
    return FMC_OK;
  });
}

// ----------------------------------------------------------- batch mode
int fmc_batch_create(const fmc_system *const *systems, int nsys, const fmc_chain_spec *chains,
                     int nchains, int precision, int guest_capacity, fmc_batch **out) {
  return guard([&] {
    if (!systems || !out) raise(FMC_ERR_ARG, "null argument");
    std::vector<const System *> sp;
    for (int i = 0; i < nsys; ++i) sp.push_back(systems[i] ? &systems[i]->s : nullptr);
    auto b = std::make_unique<fmc_batch>();
    init_chains(b->C, sp.data(), nsys, chains, nchains, precision, guest_capacity);
    // device-side pre-loading uses the system's insert0; per-chain counts
    // are applied by a system copy per distinct count
    bool custom = false;
    for (int c = 0; chains && c < nchains; ++c)
      if (chains[c].create_molecules >= 0) custom = true;
    if (custom) {
      // one SysDev per chain carrying its own insert0
      std::vector<SysDev> per(nchains);
      std::vector<ChainHdr> hh(nchains);
      FMC_CUDA(cudaMemcpy(hh.data(), b->C.hdr.p, nchains * sizeof(ChainHdr), cudaMemcpyDeviceToHost));
      for (int c = 0; c < nchains; ++c) {
        per[c] = b->C.sys[hh[c].system]->d;
        if (chains[c].create_molecules >= 0) per[c].g[0].insert0 = chains[c].create_molecules;
        hh[c].system = c;
      }
      DBuf<SysDev> tmp;
      tmp.upload(per);
      FMC_CUDA(cudaMemcpy(b->C.hdr.p, hh.data(), nchains * sizeof(ChainHdr), cudaMemcpyHostToDevice));
      std::swap(b->C.sysarr.p, tmp.p);
      std::swap(b->C.sysarr.n, tmp.n);
      b->C.launch(kModeCreate, 0);
      b->C.sync();
      std::swap(b->C.sysarr.p, tmp.p);
      std::swap(b->C.sysarr.n, tmp.n);
      for (int c = 0; c < nchains; ++c) hh[c].system = chains[c].system;
      std::vector<ChainHdr> cur(nchains);
      FMC_CUDA(cudaMemcpy(cur.data(), b->C.hdr.p, nchains * sizeof(ChainHdr), cudaMemcpyDeviceToHost));
      for (int c = 0; c < nchains; ++c) cur[c].system = chains[c].system;
      FMC_CUDA(cudaMemcpy(b->C.hdr.p, cur.data(), nchains * sizeof(ChainHdr), cudaMemcpyHostToDevice));
    } else {
      b->C.launch(kModeCreate, 0);
      b->C.sync();
    }
    b->C.check_status();
    *out = b.release();
    return FMC_OK;
  });
}

int fmc_batch_destroy(fmc_batch *b) {
  delete b;
  return FMC_OK;
}

int fmc_batch_set_log(fmc_batch *b, int cap) {
  return guard([&] {
    if (!b || cap < 0) raise(FMC_ERR_ARG, "bad argument");
    Chains &C = b->C;
    C.logcap = cap;
    C.logs.alloc(std::max(1, cap) * (size_t)C.nchains);
    C.logs.zero();
    std::vector<ChainHdr> hh(C.nchains);
    FMC_CUDA(cudaMemcpy(hh.data(), C.hdr.p, C.nchains * sizeof(ChainHdr), cudaMemcpyDeviceToHost));
    for (auto &h : hh) h.log_n = 0;
    FMC_CUDA(cudaMemcpy(C.hdr.p, hh.data(), C.nchains * sizeof(ChainHdr), cudaMemcpyHostToDevice));
    C.headers_stale = true;
    if (C.graph) {
      cudaGraphExecDestroy(C.graph);
      C.graph = nullptr;
      C.graph_moves = -1;
    }
    return FMC_OK;
  });
}

static void run_cycle(Chains &C, int nmoves) {
  if (nmoves < 0) raise(FMC_ERR_ARG, "negative move count");
  if (C.graph_moves != nmoves) {
    if (C.graph) {
      cudaGraphExecDestroy(C.graph);
      C.graph = nullptr;
    }
    cudaGraph_t g;
    FMC_CUDA(cudaStreamBeginCapture(C.stream, cudaStreamCaptureModeThreadLocal));
    C.launch(kModeMoves, nmoves);
    FMC_CUDA(cudaStreamEndCapture(C.stream, &g));
    FMC_CUDA(cudaGraphInstantiate(&C.graph, g, 0));
    cudaGraphDestroy(g);
    C.graph_moves = nmoves;
  }
  if ((int)C.host_hdr.size() != C.nchains || C.headers_stale) C.pull_headers();
  long long evals0 = 0, moves0 = 0;
  for (auto &h : C.host_hdr) {
    evals0 += h.evals;
    moves0 += h.moves;
  }
  FMC_CUDA(cudaEventRecord(C.ev0, C.stream));
  FMC_CUDA(cudaGraphLaunch(C.graph, C.stream));
  FMC_CUDA(cudaEventRecord(C.ev1, C.stream));
  C.sync();
  float ms = 0.f;
  FMC_CUDA(cudaEventElapsedTime(&ms, C.ev0, C.ev1));
  C.last_ms = ms;
  C.check_status();
  long long evals1 = 0, moves1 = 0;
  for (auto &h : C.host_hdr) {
    evals1 += h.evals;
    moves1 += h.moves;
  }
  C.last_evals = evals1 - evals0;
  C.last_moves = moves1 - moves0;
}

int fmc_batch_run(fmc_batch *b, int nmoves, fmc_chain_stats *stats) {
  return guard([&] {
    if (!b) raise(FMC_ERR_ARG, "null batch");
    run_cycle(b->C, nmoves);
    if (stats) fill_stats(b->C, stats);
    return FMC_OK;
  });
}

int fmc_batch_run_cycle(fmc_batch *b, int nmoves, const double *host_fugacity,
                        fmc_chain_stats *host_stats) {
  return guard([&] {
    if (!b) raise(FMC_ERR_ARG, "null batch");
    Chains &C = b->C;
    if (host_fugacity)  // per-chain fugacity of guest 1, applied at the cycle start
      FMC_CUDA(cudaMemcpyAsync(C.ctl_fuga.p, host_fugacity, C.nchains * sizeof(double),
                               cudaMemcpyHostToDevice, C.stream));
    run_cycle(C, nmoves);
    if (host_stats) fill_stats(C, host_stats);
    return FMC_OK;
  });
}

int fmc_batch_get_stats(fmc_batch *b, fmc_chain_stats *stats) {
  return guard([&] {
    if (!b || !stats) raise(FMC_ERR_ARG, "null argument");
    b->C.pull_headers();
    fill_stats(b->C, stats);
    return FMC_OK;
  });
}

int fmc_batch_get_log(fmc_batch *b, int chain, fmc_move_log *log, int cap, int *n) {
  return guard([&] {
    if (!b || !log || !n) raise(FMC_ERR_ARG, "null argument");
    Chains &C = b->C;
    if (chain < 0 || chain >= C.nchains) raise(FMC_ERR_ARG, "bad chain index");
    C.pull_headers();
    int m = (int)std::min<long long>(C.host_hdr[chain].log_n, std::min(cap, C.logcap));
    std::vector<LogRec> tmp(m);
    if (m)
      FMC_CUDA(cudaMemcpy(tmp.data(), C.logs.p + (size_t)chain * C.logcap, m * sizeof(LogRec),
                          cudaMemcpyDeviceToHost));
    static_assert(sizeof(LogRec) == sizeof(fmc_move_log), "log layout");
    std::memcpy(log, tmp.data(), m * sizeof(LogRec));
    *n = m;
    return FMC_OK;
  });
}

int fmc_batch_get_coords(fmc_batch *b, int chain, double *xyz, int cap, int *n) {
  return guard([&] {
    if (!b || !xyz) raise(FMC_ERR_ARG, "null argument");
    if (chain < 0 || chain >= b->C.nchains) raise(FMC_ERR_ARG, "bad chain index");
    return chain_coords(b->C, chain, 1, xyz, cap, n);
  });
}

int fmc_batch_get_coords_type(fmc_batch *b, int chain, int iguest, double *xyz, int cap, int *n) {
  return guard([&] {
    if (!b || !xyz) raise(FMC_ERR_ARG, "null argument");
    if (chain < 0 || chain >= b->C.nchains) raise(FMC_ERR_ARG, "bad chain index");
    ChainHdr hd;
    FMC_CUDA(cudaMemcpy(&hd, b->C.hdr.p + chain, sizeof hd, cudaMemcpyDeviceToHost));
    if (iguest < 1 || iguest > b->C.hsys[hd.system]->ntpguest) raise(FMC_ERR_ARG, "bad guest type");
    return chain_coords(b->C, chain, iguest, xyz, cap, n);
  });
}

int fmc_batch_get_sk(fmc_batch *b, int chain, double *sk, int cap) {
  return guard([&] {
    if (!b || !sk) raise(FMC_ERR_ARG, "null argument");
    if (chain < 0 || chain >= b->C.nchains) raise(FMC_ERR_ARG, "bad chain index");
    return chain_sk(b->C, chain, sk, cap);
  });
}

int fmc_batch_autotune(fmc_batch *b, int nmoves, int *csize_out, int nsys) {
  return guard([&] {
    if (!b) raise(FMC_ERR_ARG, "null batch");
    Chains &C = b->C;
    if (nmoves < 1) raise(FMC_ERR_ARG, "nmoves must be positive");
    if (csize_out && nsys != (int)C.sys.size())
      raise(FMC_ERR_ARG, "one cluster size per system is required");
    ChainSnapshot snap;
    save_state(C, snap);
    const long long ev0 = C.last_evals, mv0 = C.last_moves;
    const double ms0 = C.last_ms;
    C.pull_headers();
    std::vector<long long> t0(C.nchains);
    for (int c = 0; c < C.nchains; ++c) t0[c] = C.host_hdr[c].dev_ns;
    // cycle time from the saved state (best of two) and the device time of
    // every chain in that run
    auto ctrial = [&](const std::vector<int> &cc, std::vector<double> &tchain) {
      C.set_chain_clusters(cc);
      double best = 1e300;
      for (int r = 0; r < 2; ++r) {
        restore_state(C, snap);
        run_cycle(C, nmoves);
        if (C.last_ms < best) {
          best = C.last_ms;
          tchain.assign(C.nchains, 0.0);
          for (int c = 0; c < C.nchains; ++c)
            tchain[c] = 1e-6 * double(C.host_hdr[c].dev_ns - t0[c]);
        }
      }
      return best;
    };
    std::vector<int> sysof(C.nchains);
    for (int c = 0; c < C.nchains; ++c) sysof[c] = C.host_hdr[c].system;
    const int ns = (int)C.sys.size();
    auto expand = [&](const std::vector<int> &cs) {
      std::vector<int> cc(C.nchains);
      for (int c = 0; c < C.nchains; ++c) cc[c] = cs[sysof[c]];
      return cc;
    };
    // 1. per system: from one CTA per chain, double the cluster of every
    // system whose slowest chain is within 20% of the cycle, while the
    // cycle gets more than 3% faster
    std::vector<int> cs(ns, 1);
    std::vector<double> tch;
    double tcur = ctrial(expand(cs), tch);  // ctrial: per-chain times in tch
    for (;;) {
      std::vector<double> smax(ns, 0.0);
      for (int c = 0; c < C.nchains; ++c) smax[sysof[c]] = std::max(smax[sysof[c]], tch[c]);
      std::vector<int> cand = cs;
      bool changed = false;
      for (int i = 0; i < ns; ++i)
        if (smax[i] >= 0.8 * tcur && cs[i] * 2 <= kMaxCluster && C.occupancy(cs[i] * 2) >= 1) {
          cand[i] = cs[i] * 2;
          changed = true;
        }
      if (!changed) break;
      std::vector<double> t2;
      const double t = ctrial(expand(cand), t2);
      if (t >= 0.97 * tcur) break;
      cs = cand;
      tcur = t;
      tch = t2;
    }
    // (A per-chain refinement, halving light chains' clusters and doubling
    // the chains that set the cycle, won up to 1% on the trial cycle but
    // lost up to 5% on the following cycles: the heavy chains change as the
    // isotherm evolves, so the choice stays per system.)
    const std::vector<int> cur = expand(cs);
    C.set_chain_clusters(cur);
    restore_state(C, snap);
    C.last_evals = ev0;
    C.last_moves = mv0;
    C.last_ms = ms0;
    if (csize_out)  // per system: the largest cluster of its chains
      for (int i = 0; i < nsys; ++i) {
        csize_out[i] = 1;
        for (int c = 0; c < C.nchains; ++c)
          if (C.host_hdr[c].system == i) csize_out[i] = std::max(csize_out[i], cur[c]);
      }
    return FMC_OK;
  });
}

int fmc_batch_set_chain_cluster(fmc_batch *b, const int *csize, int nchains) {
  return guard([&] {
    if (!b || !csize) raise(FMC_ERR_ARG, "null argument");
    Chains &C = b->C;
    if (nchains != C.nchains) raise(FMC_ERR_ARG, "one cluster size per chain is required");
    C.set_chain_clusters(std::vector<int>(csize, csize + nchains));
    return FMC_OK;
  });
}

int fmc_batch_get_chain_cluster(const fmc_batch *b, int *csize, int nchains) {
  return guard([&] {
    if (!b || !csize) raise(FMC_ERR_ARG, "null argument");
    const Chains &C = b->C;
    if (nchains != C.nchains) raise(FMC_ERR_ARG, "one cluster size per chain is required");
    for (int c = 0; c < nchains; ++c) csize[c] = C.cchain.empty() ? 1 : C.cchain[c];
    return FMC_OK;
  });
}

int fmc_batch_save(fmc_batch *b, const char *path) {
  return guard([&] {
    if (!b || !path) raise(FMC_ERR_ARG, "null argument");
    Chains &C = b->C;
    C.sync();
    C.normalize_sk();
    std::unique_ptr<std::FILE, int (*)(std::FILE *)> f(std::fopen(path, "wb"), &std::fclose);
    if (!f) raise(FMC_ERR_ARG, std::string("cannot open ") + path);
    const int meta[6] = {C.nchains, (int)C.sys.size(), C.CA.cap, C.CA.nkmax, C.precision,
                         (int)sizeof(ChainHdr)};
    if (std::fwrite(kCkptMagic, 1, 8, f.get()) != 8 || std::fwrite(meta, sizeof meta, 1, f.get()) != 1)
      raise(FMC_ERR_ARG, "checkpoint write failed");
    ckpt_write(f.get(), C.hdr);
    ckpt_write(f.get(), C.gpos);
    ckpt_write(f.get(), C.ghi);
    ckpt_write(f.get(), C.glo);
    ckpt_write(f.get(), C.ord);
    ckpt_write(f.get(), C.freel);
    ckpt_write(f.get(), C.sk);
    ckpt_write(f.get(), C.skdf);
    ckpt_write(f.get(), C.grid);
    return FMC_OK;
  });
}

int fmc_batch_load(fmc_batch *b, const char *path) {
  return guard([&] {
    if (!b || !path) raise(FMC_ERR_ARG, "null argument");
    Chains &C = b->C;
    C.sync();
    std::unique_ptr<std::FILE, int (*)(std::FILE *)> f(std::fopen(path, "rb"), &std::fclose);
    if (!f) raise(FMC_ERR_ARG, std::string("cannot open ") + path);
    char magic[8];
    int meta[6];
    if (std::fread(magic, 1, 8, f.get()) != 8 || std::memcmp(magic, kCkptMagic, 8) != 0)
      raise(FMC_ERR_INPUT, "not a fastmc_gb300 checkpoint");
    if (std::fread(meta, sizeof meta, 1, f.get()) != 1) raise(FMC_ERR_INPUT, "checkpoint truncated");
    const int want[6] = {C.nchains, (int)C.sys.size(), C.CA.cap, C.CA.nkmax, C.precision,
                         (int)sizeof(ChainHdr)};
    if (std::memcmp(meta, want, sizeof meta) != 0)
      raise(FMC_ERR_INPUT, "checkpoint does not match this batch (chains, systems, capacity, "
                           "k-vectors, precision or library version)");
    // everything is read and checked before anything reaches the device, so
    // a rejected file leaves the batch as it was
    std::vector<ChainHdr> hdr;
    std::vector<double> gpos, grid;
    std::vector<float4> ghi, glo, skdf;
    std::vector<int> ord, freel;
    std::vector<double2> sk;
    ckpt_read(f.get(), C.hdr, hdr);
    ckpt_read(f.get(), C.gpos, gpos);
    ckpt_read(f.get(), C.ghi, ghi);
    ckpt_read(f.get(), C.glo, glo);
    ckpt_read(f.get(), C.ord, ord);
    ckpt_read(f.get(), C.freel, freel);
    ckpt_read(f.get(), C.sk, sk);
    ckpt_read(f.get(), C.skdf, skdf);
    ckpt_read(f.get(), C.grid, grid);
    validate_headers(C, hdr, ord, freel);
    ckpt_upload(C.hdr, hdr);
    ckpt_upload(C.gpos, gpos);
    ckpt_upload(C.ghi, ghi);
    ckpt_upload(C.glo, glo);
    ckpt_upload(C.ord, ord);
    ckpt_upload(C.freel, freel);
    ckpt_upload(C.sk, sk);
    ckpt_upload(C.skdf, skdf);
    ckpt_upload(C.grid, grid);
    C.headers_stale = true;
    C.pull_headers();
    return FMC_OK;
  });
}

int fmc_batch_snapshot(fmc_batch *b) {
  return guard([&] {
    if (!b) raise(FMC_ERR_ARG, "null batch");
    if (!b->snap) b->snap = std::make_unique<ChainSnapshot>();
    save_state(b->C, *b->snap);
    return FMC_OK;
  });
}

int fmc_batch_restore(fmc_batch *b) {
  return guard([&] {
    if (!b) raise(FMC_ERR_ARG, "null batch");
    if (!b->snap) raise(FMC_ERR_STATE, "no snapshot taken (fmc_batch_snapshot)");
    restore_state(b->C, *b->snap);  // the saved records select the first S(k) buffer
    return FMC_OK;
  });
}

// ------------------------------------------------------ REVIVE / REVCON
// The reference's restart files (revive, utility_pack.f:2299-2344; revread,
// gcmc.f:447-474).  REVIVE is a Fortran unformatted sequential file: each
// record is its byte count (4 bytes), the data, and the count again, as
// gfortran writes it; integers and logicals are 4 bytes, reals 8, in the
// host's byte order.  REVCON is the formatted configuration revive writes
// beside it, in CONFIG's layout.

static void frec_write(std::FILE *f, const void *p, size_t bytes) {
  if (bytes > 0x7fffffffu) raise(FMC_ERR_CAPACITY, "REVIVE record too large");
  const uint32_t n = (uint32_t)bytes;
  if (std::fwrite(&n, 4, 1, f) != 1 || (bytes && std::fwrite(p, 1, bytes, f) != bytes) ||
      std::fwrite(&n, 4, 1, f) != 1)
    raise(FMC_ERR_ARG, "REVIVE write failed");
}

static std::vector<char> frec_read(std::FILE *f, size_t want, const char *what) {
  uint32_t n = 0, m = 0;
  if (std::fread(&n, 4, 1, f) != 1) raise(FMC_ERR_INPUT, std::string("REVIVE truncated at ") + what);
  if (n != want) raise(FMC_ERR_INPUT, std::string("REVIVE record ") + what + " has the wrong length");
  std::vector<char> v(n);
  if ((n && std::fread(v.data(), 1, n, f) != n) || std::fread(&m, 4, 1, f) != 1 || m != n)
    raise(FMC_ERR_INPUT, std::string("REVIVE record ") + what + " is damaged");
  return v;
}

// Fortran edit descriptors of revive's formats, gfortran's output.
static std::string fort_e(double v, int w, int d) {  // Ew.d: 0.ddddE+xx
  char buf[64];
  int ex = 0;
  std::string digits(d, '0');
  if (v != 0.0) {
    std::snprintf(buf, sizeof buf, "%.*e", d - 1, std::fabs(v));  // m.mmmme+xx
    std::string t(buf);
    const size_t e = t.find('e');
    digits = t.substr(0, 1) + t.substr(2, e - 2);
    ex = std::atoi(t.c_str() + e + 1) + 1;
  }
  std::string out = std::string(std::signbit(v) ? "-" : "") + "0." + digits;
  char eb[16];
  if (std::abs(ex) <= 99) std::snprintf(eb, sizeof eb, "E%c%02d", ex < 0 ? '-' : '+', std::abs(ex));
  else std::snprintf(eb, sizeof eb, "%c%03d", ex < 0 ? '-' : '+', std::abs(ex));
  out += eb;
  if ((int)out.size() > w) return std::string(w, '*');
  return std::string(w - out.size(), ' ') + out;
}

static std::string fort_f(double v, int w, int d) {  // Fw.d
  char buf[128];
  std::snprintf(buf, sizeof buf, "%*.*f", w, d, v);
  std::string out(buf);
  if ((int)out.size() > w) return std::string(w, '*');
  return out;
}

static std::string fort_g(double v, int w, int d) {  // Gw.d, 4 trailing blanks in F form
  const double a = std::fabs(v);
  if (a == 0.0) return fort_f(v, w - 4, d - 1) + "    ";
  char buf[64];
  std::snprintf(buf, sizeof buf, "%.*e", d - 1, a);  // rounded to d significant digits
  const int x = std::atoi(std::strchr(buf, 'e') + 1);
  const int s = x + 1;  // digits before the decimal point of the rounded value
  if (x < -1 || s > d) return fort_e(v, w, d);
  return fort_f(v, w - 4, d - s) + "    ";
}

// The chain's guest molecule types in the reference's order, with their
// site coordinates in molecule order (molxxx/molyyy/molzzz).
struct ReviveState {
  std::vector<int> nummols;                      // [mol 1..maxmls]
  std::vector<std::vector<double>> x, y, z;      // [mol][site]
};

int fmc_batch_write_revive(fmc_batch *b, int chain, const char *dir) {
  return guard([&] {
    if (!b || !dir) raise(FMC_ERR_ARG, "null argument");
    Chains &C = b->C;
    if (chain < 0 || chain >= C.nchains) raise(FMC_ERR_ARG, "bad chain index");
    C.sync();
    C.pull_headers();
    const ChainHdr &h = C.host_hdr[chain];
    const System &s = *C.hsys[h.system];
    const int M = s.maxmls, G = s.ntpguest;
    ReviveState st;
    st.nummols.assign(M + 1, 0);
    st.x.resize(M + 1);
    st.y.resize(M + 1);
    st.z.resize(M + 1);
    for (int m = 1; m <= M; ++m) {
      const MolType &mt = s.mol[m];
      std::vector<double> xyz;
      if (mt.guest) {
        int g = 0;
        for (int i = 1; i <= G; ++i)
          if (s.locguest[i] == m) g = i;
        xyz.assign((size_t)3 * mt.natoms * std::max(1, h.nummols[g - 1]), 0.0);
        int n = 0;
        chain_coords(C, chain, g, xyz.data(), (int)xyz.size(), &n);
        st.nummols[m] = n;
        xyz.resize((size_t)3 * mt.natoms * n);
      } else {
        st.nummols[m] = mt.nummols;
        xyz = mt.xyz;
      }
      for (size_t i = 0; i < xyz.size() / 3; ++i) {
        st.x[m].push_back(xyz[3 * i]);
        st.y[m].push_back(xyz[3 * i + 1]);
        st.z[m].push_back(xyz[3 * i + 2]);
      }
    }
    int totatm = 0;
    for (int m = 1; m <= M; ++m) totatm += st.nummols[m] * s.mol[m].natoms;
    // chainstats(1 .. 16 ntpguest + 1): the production count and the open
    // window's sums (gcmc.f:1052-1077), with the moves an FP32 chain has not
    // yet added; the end-of-run averages (istat+7 .. istat+16) are zero
    // while a run goes on
    std::vector<double> cs((size_t)16 * G + 1, 0.0);
    cs[0] = double(h.prodcount);
    for (int i = 0; i < G; ++i) {
      const int mol = s.locguest[i + 1];
      const double pend = double(h.pend);
      const double dm = double((float)h.nummols[i]), e = h.energy[mol];
      const double sm = double((float)h.surfacemols[mol]);
      const double add[6] = {pend * dm, pend * e, pend * (e * dm), pend * (dm * dm), pend * (e * e),
                             pend * sm};
      for (int q = 0; q < 6; ++q) cs[1 + 16 * i + q] = h.chainstats[i][q] + add[q];
    }
    const std::string d(dir);
    {  // REVCON (utility_pack.f:2316-2326): guests first, then the framework (condense)
      std::unique_ptr<std::FILE, int (*)(std::FILE *)> f(std::fopen((d + "/REVCON").c_str(), "w"),
                                                          &std::fclose);
      if (!f) raise(FMC_ERR_ARG, "cannot open " + d + "/REVCON");
      std::string title = s.cfgname;
      title.resize(80, ' ');
      for (char &c : title)
        if ((unsigned char)c < 32) c = ' ';
      const int mol0 = s.locguest[1];
      std::string out = title + "\n" + "         0";  // levcfg 0
      char ib[32];
      std::snprintf(ib, sizeof ib, "%10d", s.imcon);
      out += ib + fort_e(h.energy[mol0], 20, 10) + "\n";
      if (s.imcon > 0)
        for (int r = 0; r < 3; ++r)
          out += fort_f(s.cell[3 * r], 20, 12) + fort_f(s.cell[3 * r + 1], 20, 12) +
                 fort_f(s.cell[3 * r + 2], 20, 12) + "\n";
      int idx = 0;
      auto emit = [&](int m) {
        const MolType &mt = s.mol[m];
        for (int k = 0; k < st.nummols[m] * mt.natoms; ++k) {
          std::string nm = mt.site[k % mt.natoms];
          nm.resize(8, ' ');
          std::snprintf(ib, sizeof ib, "%10d", ++idx);
          out += nm + ib + "\n" + fort_g(st.x[m][k], 20, 10) + fort_g(st.y[m][k], 20, 10) +
                 fort_g(st.z[m][k], 20, 10) + "\n";
        }
      };
      for (int g = 1; g <= G; ++g) emit(s.locguest[g]);
      for (int k = 1; k <= s.ntpfram; ++k) emit(s.locfram[k]);
      if (std::fwrite(out.data(), 1, out.size(), f.get()) != out.size())
        raise(FMC_ERR_ARG, "REVCON write failed");
    }
    {  // REVIVE (utility_pack.f:2328-2341)
      std::unique_ptr<std::FILE, int (*)(std::FILE *)> f(std::fopen((d + "/REVIVE").c_str(), "wb"),
                                                          &std::fclose);
      if (!f) raise(FMC_ERR_ARG, "cannot open " + d + "/REVIVE");
      const int32_t prod = h.production ? 1 : 0;
      frec_write(f.get(), &prod, 4);
      std::vector<int32_t> nm(st.nummols.begin() + 1, st.nummols.end());
      frec_write(f.get(), nm.data(), 4 * nm.size());
      frec_write(f.get(), cs.data(), 8 * cs.size());
      const int32_t na = totatm;
      frec_write(f.get(), &na, 4);
      for (int m = 1; m <= M; ++m) {
        frec_write(f.get(), st.x[m].data(), 8 * st.x[m].size());
        frec_write(f.get(), st.y[m].data(), 8 * st.y[m].size());
        frec_write(f.get(), st.z[m].data(), 8 * st.z[m].size());
      }
      // energy(i), i = 1..ntpguest, indexed by molecule type as written
      std::vector<double> en(G);
      for (int i = 1; i <= G; ++i) en[i - 1] = h.energy[i];
      frec_write(f.get(), en.data(), 8 * en.size());
    }
    return FMC_OK;
  });
}

int fmc_batch_read_revive(fmc_batch *b, int chain, const char *dir) {
  return guard([&] {
    if (!b || !dir) raise(FMC_ERR_ARG, "null argument");
    Chains &C = b->C;
    if (chain < 0 || chain >= C.nchains) raise(FMC_ERR_ARG, "bad chain index");
    C.sync();
    C.normalize_sk();
    C.pull_headers();
    const ChainHdr cur = C.host_hdr[chain];
    const System &s = *C.hsys[cur.system];
    const int M = s.maxmls, G = s.ntpguest;
    std::unique_ptr<std::FILE, int (*)(std::FILE *)> f(
        std::fopen((std::string(dir) + "/REVIVE").c_str(), "rb"), &std::fclose);
    if (!f) raise(FMC_ERR_ARG, std::string("cannot open ") + dir + "/REVIVE");
    // everything is read and checked before the chain changes
    int32_t prod = 0, na = 0;
    std::memcpy(&prod, frec_read(f.get(), 4, "production").data(), 4);
    std::vector<int32_t> nm(M);
    std::memcpy(nm.data(), frec_read(f.get(), 4 * (size_t)M, "nummols").data(), 4 * (size_t)M);
    std::vector<double> cs((size_t)16 * G + 1);
    std::memcpy(cs.data(), frec_read(f.get(), 8 * cs.size(), "chainstats").data(), 8 * cs.size());
    std::memcpy(&na, frec_read(f.get(), 4, "natms").data(), 4);
    int tot = 0;
    for (int m = 1; m <= M; ++m) {
      if (nm[m - 1] < 0) raise(FMC_ERR_INPUT, "REVIVE holds a negative molecule count");
      tot += nm[m - 1] * s.mol[m].natoms;
    }
    if (na != tot) raise(FMC_ERR_INPUT, "REVIVE's atom count does not match its molecule counts");
    std::vector<std::vector<double>> xyz(M + 1);
    for (int m = 1; m <= M; ++m) {
      const MolType &mt = s.mol[m];
      const size_t n = (size_t)nm[m - 1] * mt.natoms;
      if (!mt.guest && nm[m - 1] != mt.nummols)
        raise(FMC_ERR_INPUT, "REVIVE's framework differs from this system's");
      if (mt.guest && nm[m - 1] > C.CA.cap) raise(FMC_ERR_CAPACITY, "REVIVE exceeds the guest capacity");
      std::vector<double> c[3];
      const char *nmx[3] = {"molxxx", "molyyy", "molzzz"};
      for (int d = 0; d < 3; ++d) {
        c[d].resize(n);
        if (n) std::memcpy(c[d].data(), frec_read(f.get(), 8 * n, nmx[d]).data(), 8 * n);
        else frec_read(f.get(), 0, nmx[d]);
      }
      xyz[m].resize(3 * n);
      for (size_t i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) xyz[m][3 * i + d] = c[d][i];
      if (!mt.guest)  // the framework is the system's (frozen; its tables are built)
        for (size_t i = 0; i < 3 * n; ++i)
          if (std::fabs(xyz[m][i] - mt.xyz[i]) > 1e-9)
            raise(FMC_ERR_INPUT, "REVIVE's framework differs from this system's");
    }
    frec_read(f.get(), 8 * (size_t)G, "energy");  // single_point recomputes the energies
    // a new chain record as the start-up leaves it (production from
    // eqsteps, gcmc.f:450-465, 600), keeping the chain's generator, pressure,
    // log and device time; the open window's sums from the file
    ChainHdr h = initial_header(s, cur.system, 0, nullptr);
    std::memcpy(h.u, cur.u, sizeof h.u);
    h.c = cur.c;
    h.cd = cur.cd;
    h.cm = cur.cm;
    h.ir = cur.ir;
    h.jr = cur.jr;
    std::memcpy(h.rbuf, cur.rbuf, sizeof h.rbuf);
    h.rhead = cur.rhead;
    h.ravail = cur.ravail;
    std::memcpy(h.fuga, cur.fuga, sizeof h.fuga);
    h.log_n = cur.log_n;
    h.dev_ns = cur.dev_ns;
    FMC_CUDA(cudaMemcpy(C.hdr.p + chain, &h, sizeof h, cudaMemcpyHostToDevice));
    const size_t so = (size_t)chain * kMaxG * C.CA.nkmax;
    if (C.sk.p) FMC_CUDA(cudaMemset(C.sk.p + so, 0, sizeof(double2) * kMaxG * C.CA.nkmax));
    if (C.skdf.p) FMC_CUDA(cudaMemset(C.skdf.p + so, 0, sizeof(float4) * kMaxG * C.CA.nkmax));
    if (C.skdf2.p) FMC_CUDA(cudaMemset(C.skdf2.p + so, 0, sizeof(float4) * kMaxG * C.CA.nkmax));
    if (C.grid.p)  // probability grids start again with the run
      FMC_CUDA(cudaMemset(C.grid.p + (size_t)chain * C.CA.grid_stride, 0,
                          sizeof(double) * C.CA.grid_stride));
    // the molecules, each type in order, inserted where they are
    for (int g = 1; g <= G; ++g) {
      const int m = s.locguest[g];
      const int n = nm[m - 1];
      if (n == 0) continue;
      DBuf<double> in;
      in.upload(xyz[m]);
      WidomJob wj{};
      wj.chain = chain;
      wj.iguest = g - 1;
      wj.ntrial = n;
      wj.nstep = 1;
      wj.ng[0] = wj.ng[1] = wj.ng[2] = 1;
      wj.xyz_in = in.p;
      FMC_CUDA(C.launch_one(1, 1, nullptr, C.stream, kModeLoad, 0, wj));
      C.sync();
    }
    C.headers_stale = true;
    C.pull_headers();
    ChainHdr &hn = C.host_hdr[chain];
    if (hn.status) raise(FMC_ERR_DEVICE, "loading the REVIVE molecules raised a device status");
    for (int i = 0; i < G; ++i)
      for (int q = 0; q < 6; ++q) hn.chainstats[i][q] = cs[1 + 16 * i + q];
    FMC_CUDA(cudaMemcpy(C.hdr.p + chain, &hn, sizeof hn, cudaMemcpyHostToDevice));
    (void)prod;  // revread's production flag gives way to eqsteps at start-up
    return FMC_OK;
  });
}

// Widom test insertions (widom_grid, gcmc.f:2454-2548) on one chain: one
// CTA per SM, each taking every gridDim-th trial against the chain's state,
// which no trial changes.
static void run_widom(Chains &C, WidomJob wj, int ns, double *henry, int64_t *counts,
                      double *estep_out, int *overlap_out, double *xyz_out) {
  if (wj.ntrial < 1) raise(FMC_ERR_ARG, "no trial insertions");
  int dev = 0, nsm = 1;
  FMC_CUDA(cudaGetDevice(&dev));
  FMC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int grid = std::min(wj.ntrial, nsm);
  DBuf<double> partial, est, xyz;
  DBuf<int> ovl;
  partial.alloc((size_t)grid * 3);
  if (estep_out) est.alloc(wj.ntrial);
  if (overlap_out) ovl.alloc(wj.ntrial);
  if (xyz_out) xyz.alloc((size_t)wj.ntrial * ns * 3);
  wj.partial = partial.p;
  wj.estep_out = est.p;
  wj.overlap_out = ovl.p;
  wj.xyz_out = xyz.p;
  FMC_CUDA(C.launch_one(grid, 1, nullptr, C.stream, kModeWidom, 0, wj));
  C.sync();
  std::vector<double> part((size_t)grid * 3);
  FMC_CUDA(cudaMemcpy(part.data(), partial.p, part.size() * sizeof(double), cudaMemcpyDeviceToHost));
  double sum = 0.0, nok = 0.0, ntot = 0.0;
  for (int i = 0; i < grid; ++i) {
    if (part[3 * i + 2] < 0.0)
      raise(FMC_ERR_DEVICE, "a Widom trial raised a device status (table range, segments)");
    sum += part[3 * i];
    nok += part[3 * i + 1];
    ntot += part[3 * i + 2];
  }
  // gcmc.f:2544-2545: averaged over every trial, overlapping ones included
  if (henry) *henry = ntot > 0 ? sum / ntot : 0.0;
  if (counts) {
    counts[0] = (int64_t)nok;
    counts[1] = (int64_t)ntot;
  }
  if (estep_out)
    FMC_CUDA(cudaMemcpy(estep_out, est.p, wj.ntrial * sizeof(double), cudaMemcpyDeviceToHost));
  if (overlap_out)
    FMC_CUDA(cudaMemcpy(overlap_out, ovl.p, wj.ntrial * sizeof(int), cudaMemcpyDeviceToHost));
  if (xyz_out)
    FMC_CUDA(cudaMemcpy(xyz_out, xyz.p, (size_t)wj.ntrial * ns * 3 * sizeof(double),
                        cudaMemcpyDeviceToHost));
}

static int widom_guest(const Chains &C, int chain, int iguest, int *ns) {
  if (chain < 0 || chain >= C.nchains) raise(FMC_ERR_ARG, "bad chain index");
  const ChainHdr &h = C.host_hdr[chain];
  const System &s = *C.hsys[h.system];
  if (iguest < 1 || iguest > s.ntpguest) raise(FMC_ERR_ARG, "bad guest type");
  *ns = s.mol[s.locguest[iguest]].natoms;
  return h.system;
}

int fmc_widom_grid(fmc_batch *b, int chain, int iguest, const int *ngrid, int nstep, int64_t seed,
                   double *henry, int64_t *counts, double *estep_out, int *overlap_out,
                   double *xyz_out) {
  return guard([&] {
    if (!b || !ngrid) raise(FMC_ERR_ARG, "null argument");
    Chains &C = b->C;
    if (C.headers_stale || (int)C.host_hdr.size() != C.nchains) C.pull_headers();
    int ns = 0;
    widom_guest(C, chain, iguest, &ns);
    if (ngrid[0] < 1 || ngrid[1] < 1 || ngrid[2] < 1 || nstep < 1) raise(FMC_ERR_ARG, "empty grid");
    const long long nt = (long long)ngrid[0] * ngrid[1] * ngrid[2] * nstep;
    if (nt > (1LL << 31) - 1) raise(FMC_ERR_ARG, "too many trials in one call");
    WidomJob wj{};
    wj.chain = chain;
    wj.iguest = iguest - 1;
    wj.ntrial = (int)nt;
    wj.nstep = nstep;
    for (int d = 0; d < 3; ++d) wj.ng[d] = ngrid[d];
    wj.seed = (unsigned long long)seed;
    run_widom(C, wj, ns, henry, counts, estep_out, overlap_out, xyz_out);
    return FMC_OK;
  });
}

int fmc_batch_prob_info(fmc_batch *b, int chain, int *ngrid, int *nsub) {
  return guard([&] {
    if (!b || !ngrid || !nsub) raise(FMC_ERR_ARG, "null argument");
    Chains &C = b->C;
    if (chain < 0 || chain >= C.nchains) raise(FMC_ERR_ARG, "chain out of range");
    C.pull_headers();
    const System &s = *C.hsys[C.host_hdr[chain].system];
    for (int d = 0; d < 3; ++d) ngrid[d] = s.lprob ? s.ngrid[d] : 0;
    *nsub = s.lprob ? s.ntprob : 0;
    return FMC_OK;
  });
}

int fmc_batch_prob_grid(fmc_batch *b, int chain, int sub, double *out, int64_t n) {
  return guard([&] {
    if (!b || !out) raise(FMC_ERR_ARG, "null argument");
    Chains &C = b->C;
    if (chain < 0 || chain >= C.nchains) raise(FMC_ERR_ARG, "chain out of range");
    C.pull_headers();
    const System &s = *C.hsys[C.host_hdr[chain].system];
    if (!s.lprob || sub < 0 || sub >= s.ntprob) raise(FMC_ERR_ARG, "no such probability grid");
    const int64_t gs = (int64_t)s.ngrid[0] * s.ngrid[1] * s.ngrid[2];
    if (n < gs) raise(FMC_ERR_ARG, "output buffer too small");
    C.sync();
    FMC_CUDA(cudaMemcpy(out, C.grid.p + (size_t)chain * C.CA.grid_stride + (size_t)sub * gs,
                        gs * sizeof(double), cudaMemcpyDeviceToHost));
    return FMC_OK;
  });
}

int fmc_widom_positions(fmc_batch *b, int chain, int iguest, int npos, const double *xyz,
                        double *estep_out, int *overlap_out) {
  return guard([&] {
    if (!b || !xyz) raise(FMC_ERR_ARG, "null argument");
    Chains &C = b->C;
    if (C.headers_stale || (int)C.host_hdr.size() != C.nchains) C.pull_headers();
    int ns = 0;
    widom_guest(C, chain, iguest, &ns);
    if (npos < 1) raise(FMC_ERR_ARG, "no positions");
    DBuf<double> in;
    in.upload(std::vector<double>(xyz, xyz + (size_t)npos * ns * 3));
    WidomJob wj{};
    wj.chain = chain;
    wj.iguest = iguest - 1;
    wj.ntrial = npos;
    wj.nstep = 1;
    wj.ng[0] = wj.ng[1] = wj.ng[2] = 1;
    wj.xyz_in = in.p;
    run_widom(C, wj, ns, nullptr, nullptr, estep_out, overlap_out, nullptr);
    return FMC_OK;
  });
}

int fmc_batch_set_cluster(fmc_batch *b, const int *csize, int nsys) {
  return guard([&] {
    if (!b || !csize) raise(FMC_ERR_ARG, "null argument");
    Chains &C = b->C;
    if (nsys != (int)C.sys.size()) raise(FMC_ERR_ARG, "one cluster size per system is required");
    C.set_clusters(std::vector<int>(csize, csize + nsys));
    return FMC_OK;
  });
}

int fmc_batch_set_speculation(fmc_batch *b, int kmax) {
  return guard([&] {
    if (!b) raise(FMC_ERR_ARG, "null batch");
    if (kmax < 0 || kmax > kMaxSpec) raise(FMC_ERR_ARG, "kmax must be 0..8");
    Chains &C = b->C;
    C.CA.spec_max = kmax;
    if (C.graph) {  // the launches captured the old value
      cudaGraphExecDestroy(C.graph);
      C.graph = nullptr;
    }
    C.graph_moves = -1;
    return FMC_OK;
  });
}

int fmc_batch_get_cluster(const fmc_batch *b, int *csize, int nsys) {
  return guard([&] {
    if (!b || !csize) raise(FMC_ERR_ARG, "null argument");
    const Chains &C = b->C;
    if (nsys != (int)C.sys.size()) raise(FMC_ERR_ARG, "one cluster size per system is required");
    if (!C.csys.empty()) {
      for (int i = 0; i < nsys; ++i) csize[i] = C.csys[i];
    } else {  // per-chain sizes: the largest of each system's chains
      std::vector<ChainHdr> hh(C.nchains);
      FMC_CUDA(cudaMemcpy(hh.data(), C.hdr.p, C.nchains * sizeof(ChainHdr), cudaMemcpyDeviceToHost));
      for (int i = 0; i < nsys; ++i) csize[i] = 1;
      for (int c = 0; c < C.nchains && !C.cchain.empty(); ++c)
        csize[hh[c].system] = std::max(csize[hh[c].system], C.cchain[c]);
    }
    return FMC_OK;
  });
}

int fmc_batch_last_timing(const fmc_batch *b, double *kernel_ms, int64_t *evals, int64_t *moves) {
  return guard([&] {
    if (!b) raise(FMC_ERR_ARG, "null batch");
    if (kernel_ms) *kernel_ms = b->C.last_ms;
    if (evals) *evals = b->C.last_evals;
    if (moves) *moves = b->C.last_moves;
    return FMC_OK;
  });
}

// Same result and side effect as fmc_full_ewald, with no device allocation:
// the kernels read the guests where the chain keeps them and use the static
// scratch above.  Limit: newld <= 65528 k-vectors (FMC_ERR_ARG beyond).
int fmc_full_ewald_noalloc(fmc_plain *h, double *out4) {
  return guard([&] {
    if (!h || !out4) raise(FMC_ERR_ARG, "null argument");
    Chains &C = h->C;
    C.normalize_sk();
    const System &s = *C.hsys[0];
    const DevSystem &D = *C.sys[0];
    const int nk = s.newld;
    const int nb = (nk + kKB - 1) / kKB;
    if (nb + 1 > kNoallocScratchDoubles) {
      char buf[256];
      std::snprintf(buf, sizeof buf,
                    "fmc_full_ewald_noalloc: %d k-vectors need %d partial sums but its static "
                    "scratch holds %d (at most %d k-vectors); use fmc_full_ewald",
                    nk, nb, kNoallocScratchDoubles - 1, (kNoallocScratchDoubles - 1) * kKB);
      raise(FMC_ERR_ARG, buf);
    }
    if (s.ntpguest > kMaxG) raise(FMC_ERR_ARG, "too many guest types");
    int cur = -1;
    FMC_CUDA(cudaGetDevice(&cur));
    if (cur != C.device)
      raise(FMC_ERR_ARG, "fmc_full_ewald_noalloc: call with device " + std::to_string(C.device) +
                             " (the engine's) current, not device " + std::to_string(cur));
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    double *scr = noalloc_scratch();
    // guest counts and system charge of chain 0, straight from its header
    static_assert(sizeof(ChainHdr::nummols) == sizeof(int) * kMaxG, "nummols layout");
    static_assert(std::is_same<decltype(ChainHdr::sumchg), double>::value, "sumchg type");
    int nummols[kMaxG] = {};
    double sumchg = 0.0;
    const char *hdr0 = reinterpret_cast<const char *>(C.hdr.p);
    FMC_CUDA(cudaMemcpyAsync(nummols, hdr0 + offsetof(ChainHdr, nummols), sizeof nummols,
                             cudaMemcpyDeviceToHost, C.stream));
    FMC_CUDA(cudaMemcpyAsync(&sumchg, hdr0 + offsetof(ChainHdr, sumchg), sizeof sumchg,
                             cudaMemcpyDeviceToHost, C.stream));
    C.sync();
    GuestSites gs{};
    gs.ntp = s.ntpguest;
    double sq = 0.0, e3 = 0.0;
    const MolType &fw = s.mol[s.fw_mol];
    for (int m = 0; m < fw.nummols; ++m)
      for (int i = 0; i < fw.natoms; ++i) sq += fw.chg[i] * fw.chg[i];
    for (int g = 0; g < s.ntpguest; ++g) {
      const MolType &gm = s.mol[s.locguest[g + 1]];
      if (gm.natoms > kMaxS) raise(FMC_ERR_ARG, "too many guest sites");
      if (nummols[g] < 0 || nummols[g] > C.CA.cap) raise(FMC_ERR_DEVICE, "guest count out of range");
      gs.n[g] = nummols[g];
      gs.ns[g] = gm.natoms;
      for (int i = 0; i < gm.natoms; ++i) gs.q[g][i] = gm.chg[i];
      for (int m = 0; m < nummols[g]; ++m)
        for (int i = 0; i < gm.natoms; ++i) sq += gm.chg[i] * gm.chg[i];
      e3 += nummols[g] * s.ewald3en[s.locguest[g + 1]];
    }
    double eng = 0.0;
    if (nk > 0) {
      Rcell rc;
      for (int i = 0; i < 9; ++i) rc.r[i] = D.d.rcell[i];
      const bool f32 = C.precision == FMC_PREC_FP32;
      guest_ewald_kernel<<<nb, kThreads, 0, C.stream>>>(
          C.gpos.p, C.ord.p, C.CA.cap, gs, D.klmn.p, nk, rc, D.akk.p, D.skfw.p,
          f32 ? nullptr : C.sk.p, f32 ? C.skdf.p : nullptr, C.CA.nkmax, scr);
      FMC_CUDA(cudaGetLastError());
      partial_sum_kernel<<<1, kThreads, 0, C.stream>>>(scr, nb, scr + nb);
      FMC_CUDA(cudaGetLastError());
      FMC_CUDA(cudaMemcpyAsync(&eng, scr + nb, sizeof eng, cudaMemcpyDeviceToHost, C.stream));
      C.sync();
    }
    const double r4 = fmc::kR4pie0 / s.epsq;
    const double sic = -r4 * s.alpha * sq / fmc::kSqrPi;
    const double qfix = -(0.5 * fmc::kPi * r4) * ((sumchg / s.alpha) * (sumchg / s.alpha) / s.volm);
    const double ew1 = 2.0 * (2.0 * fmc::kPi / s.volm) * r4 * eng + sic + qfix;
    out4[0] = (ew1 - e3) / s.engunit;
    out4[1] = ew1;
    out4[2] = sic;
    out4[3] = qfix;
    return FMC_OK;
  });
}

int fmc_batch_cycle_bytes(const fmc_batch *b, int64_t *h2d, int64_t *d2h) {
  return guard([&] {
    if (!b) raise(FMC_ERR_ARG, "null batch");
    if (h2d) *h2d = (int64_t)b->C.nchains * (int64_t)sizeof(double);
    if (d2h) *d2h = (int64_t)b->C.nchains * (int64_t)sizeof(ChainHdr);
    return FMC_OK;
  });
}

}  // extern "C"

// device_eval.cuh -- cooperative evaluation of the guest energy at one or two
// positions (the new and, for displacements, the old one).
//
// Restates, per CTA:
//   guestlistgen + images + surface_check (utility_pack.f:3711-3774,
//     1697-1791; mc_moves.f:10-44): neighbour search by cell columns,
//     minimum image by the column's periodic shift, overlap and surface
//     flags;
//   ewald2 (ewald.f:663-733) and srfrce (vdw_terms.f:382-466): tabulated
//     erfc and van der Waals terms with the reference's 3-point
//     interpolation (FP64 path) or the same quadratic written as
//     A + p(B + pC) with FP64-built FP32 coefficients (FP32 path);
//   ewald1_guest (ewald.f:32-352): per-k structure factor of the guest,
//     its energy against S(k) and the per-molecule-type mixing terms
//     (engine.cuh).
//
// The FP32 path keeps distances accurate to about one FP32 rounding of r:
// coordinates are float hi/lo pairs and periodic shifts are applied with
// error-free sums, so no FP64 instruction runs per pair.
#pragma once

#include "device_core.cuh"

namespace fmcdev {

// Near molecules one CTA lists per evaluated position (resident guests).
constexpr int kGList = 2 * kThreads;

template <bool F32>
struct EvalSmem {
  double p64[2][kMaxS][3];
  float phi[2][kMaxS][3];
  float plo[2][kMaxS][3];
  // power tables e^{i 2 pi j s_d}: [pos][site][axis][j]
  double2 pw64[F32 ? 1 : 2][F32 ? 1 : kMaxS][3][F32 ? 1 : kMaxKm];
  float2 pw32[F32 ? 2 : 1][F32 ? kMaxS : 1][3][F32 ? kMaxKm : 1];
  // FP32 path: e^{i 2 pi (l s_x + m s_y)} per position and site, indexed
  // [(p * ns + s) * nlm + l * (2 kmax_y + 1) + m + kmax_y], when it fits
  float2 plm[F32 ? kPlmMax : 1];
  float fhi[2][kMaxS][3];   // fractional coordinates as float hi/lo pairs
  float flo[2][kMaxS][3];
  float cen[2][3];          // centre and bounding radius of each position
  float rmx[2];
  int seg_start[kMaxSeg];
  int seg_pref[kMaxSeg + 1];
  int seg_shift[kMaxSeg];
  int nslots;
  // FP32 path, resident guests: molecules near the evaluated position
  int glist[F32 ? kGList : 1];
  int gcount;
  int rank, csize;          // this CTA's place in the chain's cluster
  // positions the (l, m) table is sized for when deciding whether it is
  // used: 2 wherever S(k) is committed, so that a site's s(k) comes out of
  // the same arithmetic whether one or two positions are evaluated and the
  // running S(k) stays the exact sum of its molecules' terms; 1 for Widom
  // trials, which commit nothing
  int tabpos;
  int red_i[kWarps + 1];
  double red[kWarps * 32];
  double out[64];
};

// -------------------------------------------------------------- pair terms
// FP64 3-point interpolation (ewald.f:703-715, vdw_terms.f:441-453).
__device__ __forceinline__ double interp64(const double *tab, double r, double rd,
                                           int mx, int &st) {
  double t = r * rd;
  int l = int(t);
  if (l < 1 || l + 2 > mx + 2) {
    st |= kStTableLow;
    return 0.0;
  }
  double p = t - double(l);
  double v0 = __ldg(tab + l), v1 = __ldg(tab + l + 1), v2 = __ldg(tab + l + 2);
  double t1 = v0 + (v1 - v0) * p;
  double t2 = v1 + (v2 - v1) * (p - 1.0);
  return t1 + (t2 - t1) * p * 0.5;
}

// FP32 form: index from r*rd with the product's rounding error recovered
// by an FMA, value A + p(B + pC).
__device__ __forceinline__ float interp32(const float4 *tab, float r, float rd,
                                          int mx, int &st) {
  float t = r * rd;
  float e = fmaf(r, rd, -t);
  int l = int(t);
  if (l < 1 || l + 2 > mx + 2) {
    st |= kStTableLow;
    return 0.0f;
  }
  float p = (t - float(l)) + e;
  float4 c = __ldg(tab + l);
  return fmaf(p, fmaf(p, c.z, c.y), c.x);
}

struct SiteInfo {
  double q;      // site charge
  double chgea;  // q / epsq * r4pie0
  float chgeaf;  // chgea as an FP32 hi/lo pair
  float chgeaf_lo;
  float qf;
  int type;
  const int *prow;     // table row per partner atom type (the guest type's record)
  const float *psig2;  // surface distance squared per partner atom type
};

// One site-atom pair: erfc and van der Waals terms when r < rc, overlap and
// surface flags like surface_check.
__device__ __forceinline__ void pair_term64(const SysDev &S, const SiteInfo &si, double qb,
                                            int tb, int frozen_b, double r2, double &e2,
                                            double &vdw, int &ov, int &sf, int &st) {
  int pi = si.type * (S.ntpatm + 1) + tb;
  if (r2 < S.overlap_sq) ov = 1;
  if (frozen_b && r2 < __ldg(S.sig2 + pi)) sf = 1;
  if (r2 < S.rc2) {
    double r = sqrt(r2);
    double chgprd = si.chgea * qb;
    if (fabs(chgprd) > 1.0e-10) e2 += interp64(S.erc, r, S.rdrewd, S.mxegrd, st) * chgprd;
    int k = __ldg(S.pairtab + pi);
    if (k >= 0) vdw += interp64(S.vvv + (size_t)k * S.tabstride, r, S.rdlrpot, S.mxegrd, st);
  }
}

// FP32 path.  The erfc term is formed and summed as a hi/lo pair: the
// charge product (site factor and atom charge both as pairs), the table
// value A + A_lo + p(B + pC) and the product's FMA residual, so each term
// keeps about 1e-9 of its value apart from the FP32 distance.
__device__ __forceinline__ void pair_term32(const SysDev &S, const SiteInfo &si, float qh, float ql,
                                            int tb, int frozen_b, float r2, AccT<true> &e2,
                                            float &vdw, int &ov, int &sf, int &st,
                                            bool skip_vdw = false) {
  if (r2 < S.overlap_sqf) ov = 1;
  if (frozen_b && r2 < si.psig2[tb]) sf = 1;
  if (r2 < S.rc2f) {
    float r = sqrtf(r2);
    const float ch = si.chgeaf * qh;
    if (fabsf(ch) > 1.0e-10f) {
      const float cl = fmaf(si.chgeaf, qh, -ch) + fmaf(si.chgeaf, ql, si.chgeaf_lo * qh);
      float t = r * S.rdrewdf;
      float e = fmaf(r, S.rdrewdf, -t);
      int l = int(t);
      if (l < 1 || l > S.mxegrd) {
        st |= kStTableLow;
      } else {
        float p = (t - float(l)) + e;
        float4 c = __ldg(S.ercq + l);
        float vl = fmaf(p, fmaf(p, c.z, c.y), c.w);
        float ph = c.x * ch;
        float pl = fmaf(c.x, ch, -ph) + fmaf(c.x, cl, vl * ch);
        e2.add_df(DF{ph, pl});
      }
    }
    const int k = si.prow[tb];
    if (k >= 0 && !skip_vdw) vdw += interp32(S.vvvq + (size_t)k * S.tabstride, r, S.rdlrpotf, S.mxegrd, st);
  }
}

// Close pairs: below 3 A the Lennard-Jones table is steep enough (tens of
// thousands of kcal/mol per A near the overlap distance) that an FP32
// distance alone would cost ~1e-6 of the term.  These pairs take r^2, r,
// the bin index r*rdlrpot and the table value as float hi/lo pairs.
constexpr float kNear2 = 9.0f;

__device__ __forceinline__ bool vdw_is_near(const SysDev &S, const SiteInfo &si, int tb, float r2) {
  return r2 < kNear2 && si.prow[tb] >= 0;
}

// Lennard-Jones term of one close pair from the difference vector given as
// hi/lo pairs per axis.
__device__ __forceinline__ DF vdw_near_df(const SysDev &S, const SiteInfo &si, int tb,
                                          const float *dh, const float *dl, int &st) {
  float ph[3], pe[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    ph[d] = dh[d] * dh[d];
    pe[d] = fmaf(dh[d], dh[d], -ph[d]) + 2.0f * dh[d] * dl[d];
  }
  float s1, e1, s2, e2;
  two_sum_f(ph[0], ph[1], s1, e1);
  two_sum_f(s1, ph[2], s2, e2);
  const float r2l = (e1 + e2) + (pe[0] + pe[1] + pe[2]);
  const float rh = sqrtf(s2);
  const float rl = (fmaf(-rh, rh, s2) + r2l) * (0.5f / rh);
  const float th = rh * S.rdlrpotf;
  const float tl = fmaf(rh, S.rdlrpotf, -th) + fmaf(rh, S.rdlrpotf_lo, rl * S.rdlrpotf);
  int l = (int)floorf(th);
  float p = (th - (float)l) + tl;
  if (p < 0.0f) {
    l -= 1;
    p += 1.0f;
  } else if (p >= 1.0f) {
    l += 1;
    p -= 1.0f;
  }
  DF out{0.0f, 0.0f};
  if (l < 1 || l > S.mxegrd) {
    st |= kStTableLow;
    return out;
  }
  const int k = si.prow[tb];
  const float4 c = __ldg(S.vvvq + (size_t)k * S.tabstride + l);
  const float q = fmaf(p, fmaf(p, c.z, c.y), c.w);  // A_lo + p(B + pC)
  two_sum_f(c.x, q, out.hi, out.lo);
  return out;
}

// Minimum-image difference p - q of two points given as float hi/lo pairs
// (one axis).  The image shift is applied with an error-free sum so the
// result keeps the relative accuracy of a single FP32 subtraction.
__device__ __forceinline__ float mi_diff32(float ph, float pl, float qh, float ql, float Lh,
                                           float Ll, float rL) {
  float dh = ph - qh;
  float k = rint_image(dh * rL);
  if (k != 0.0f) {
    float h, e;
    two_sum_f(ph, -k * Lh, h, e);
    return (h - qh) + ((pl - ql) + (e - k * Ll));
  }
  return dh + (pl - ql);
}

// The same difference as a hi/lo pair (close pairs).
__device__ __forceinline__ void mi_diff_df(float ph, float pl, float qh, float ql, float Lh,
                                           float Ll, float rL, float &dh, float &dl) {
  float k = rint_image((ph - qh) * rL);
  float a = ph, al = pl;
  if (k != 0.0f) {
    float h, e;
    two_sum_f(ph, -k * Lh, h, e);
    a = h;
    al = pl + (e - k * Ll);
  }
  float s, e;
  two_sum_f(a, -qh, s, e);
  dh = s;
  dl = e + (al - ql);
}

// Parallelepiped cells (imcon 3): the minimum image of p - q for points as
// float hi/lo pairs.  images (utility_pack.f:1697-1902, imcon 3) takes the
// fractional difference s = rcell d, removes nint(s) and goes back through
// the cell; here the same image, the integer cell translation n =
// nint(rcell d), is taken off as d - cell n with the cell edges as hi/lo
// pairs and exact products, so the difference keeps the accuracy of its
// hi/lo inputs (the FP32 rounding of rcell d only matters for points half
// a cell apart, far beyond any cutoff).
__device__ __forceinline__ void mi_tric_df(const SysDev &S, const float *ph, const float *pl,
                                           const float *qh, const float *ql, float *dh,
                                           float *dl) {
  float d0[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) d0[j] = (ph[j] - qh[j]) + (pl[j] - ql[j]);
  float n[3];
#pragma unroll
  for (int k = 0; k < 3; ++k)
    n[k] = rintf(fmaf(S.rcellh[k], d0[0], fmaf(S.rcellh[k + 3], d0[1], S.rcellh[k + 6] * d0[2])));
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    float th = 0.f, tl = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (n[k] != 0.f) {
        const float c = S.cellh[j + 3 * k];
        const float p = n[k] * c;
        const float pe = fmaf(n[k], c, -p) + n[k] * S.celll[j + 3 * k];
        float s, e;
        two_sum_f(th, p, s, e);
        th = s;
        tl += e + pe;
      }
    }
    float s1, e1, s2, e2;
    two_sum_f(ph[j], -qh[j], s1, e1);
    two_sum_f(s1, -th, s2, e2);
    dh[j] = s2;
    dl[j] = (e1 + e2) + ((pl[j] - ql[j]) - tl);
  }
}

// Plain FP32 minimum image of a difference vector in a parallelepiped cell
// (prefilters: accurate to about 1e-6 A), r^2.
__device__ __forceinline__ float tric_r2_f32(const SysDev &S, float dx, float dy, float dz) {
  float n[3];
#pragma unroll
  for (int k = 0; k < 3; ++k)
    n[k] = rintf(fmaf(S.rcellh[k], dx, fmaf(S.rcellh[k + 3], dy, S.rcellh[k + 6] * dz)));
  const float *c = S.cellh;
  dx -= fmaf(c[0], n[0], fmaf(c[3], n[1], c[6] * n[2]));
  dy -= fmaf(c[1], n[0], fmaf(c[4], n[1], c[7] * n[2]));
  dz -= fmaf(c[2], n[0], fmaf(c[5], n[1], c[8] * n[2]));
  return fmaf(dx, dx, fmaf(dy, dy, dz * dz));
}

// The same as one float per axis, and r^2.
__device__ __forceinline__ float mi_tric_r2(const SysDev &S, const float *ph, const float *pl,
                                            const float *qh, const float *ql) {
  float dh[3], dl[3];
  mi_tric_df(S, ph, pl, qh, ql, dh, dl);
  const float x = dh[0] + dl[0], y = dh[1] + dl[1], z = dh[2] + dl[2];
  return fmaf(x, x, fmaf(y, y, z * z));
}

__device__ __forceinline__ int image_of(int ic, int n) {
  return (ic >= 0) ? ic / n : -((-ic + n - 1) / n);
}

// ---------------------------------------------------- framework neighbours
// List of framework atom segments (runs of cells along z in one column and
// one periodic image) covering the sphere of radius R around c.  On a
// cluster each CTA takes every csize-th column.  Slots with
// zero atoms are allowed; seg_pref is the prefix over slots.  The geometry
// is conservative (FP32 with a margin): it only selects candidates.
template <bool F32>
__device__ void build_segments(const SysDev &S, EvalSmem<F32> &sm, const float *c, float R,
                               int &st) {
  if (!S.use_cells) {  // every framework atom, this CTA's share of a cluster
    if (threadIdx.x == 0) {
      int a0, a1;
      share_of(S.nfw, sm.rank, sm.csize, a0, a1);
      sm.seg_start[0] = a0;
      sm.seg_shift[0] = (2) | (2 << 4) | (2 << 8);
      sm.seg_pref[0] = 0;
      sm.seg_pref[1] = a1 - a0;
      sm.nslots = 1;
    }
    __syncthreads();
    return;
  }
  const float *cs = S.cszf, *rc = S.rcszf;
  int ix0 = (int)floorf((c[0] - R) * rc[0]), ix1 = (int)floorf((c[0] + R) * rc[0]);
  int iy0 = (int)floorf((c[1] - R) * rc[1]), iy1 = (int)floorf((c[1] + R) * rc[1]);
  int nx = ix1 - ix0 + 1, ny = iy1 - iy0 + 1;
  int ncol = nx * ny;
  const int kRuns = 4;
  int nslot = ncol * kRuns;
  if (nslot > kMaxSeg) {
    if (threadIdx.x == 0) {
      st |= kStSegOverflow;
      sm.nslots = 0;
      sm.seg_pref[0] = 0;
    }
    __syncthreads();
    return;
  }
  float R2 = R * R;
  for (int col = threadIdx.x; col < ncol; col += kThreads) {
    int ix = ix0 + col / ny, iy = iy0 + col % ny;
    float xlo = ix * cs[0], xhi = xlo + cs[0];
    float ylo = iy * cs[1], yhi = ylo + cs[1];
    float dx = fmaxf(0.f, fmaxf(xlo - c[0], c[0] - xhi));
    float dy = fmaxf(0.f, fmaxf(ylo - c[1], c[1] - yhi));
    float d2 = dx * dx + dy * dy;
    int base = col * kRuns;
    for (int r = 0; r < kRuns; ++r) {
      sm.seg_start[base + r] = 0;
      sm.seg_shift[base + r] = 0;
      sm.seg_pref[base + r] = 0;  // count for now
    }
    if (d2 > R2) continue;
    if (col % sm.csize != sm.rank) continue;  // another CTA of the cluster takes this column
    float hz = sqrtf(R2 - d2);
    int iz0 = (int)floorf((c[2] - hz) * rc[2]), iz1 = (int)floorf((c[2] + hz) * rc[2]);
    int imx = image_of(ix, S.nc[0]), imy = image_of(iy, S.nc[1]);
    int ixw = ix - imx * S.nc[0], iyw = iy - imy * S.nc[1];
    int colbase = (ixw * S.nc[1] + iyw) * S.nc[2];
    int r = 0;
    int iz = iz0;
    while (iz <= iz1) {
      int imz = image_of(iz, S.nc[2]);
      int izw = iz - imz * S.nc[2];
      int run_end = min(iz1, (imz + 1) * S.nc[2] - 1);
      int izw_end = run_end - imz * S.nc[2];
      if (r >= kRuns || imx < -2 || imx > 2 || imy < -2 || imy > 2 || imz < -2 || imz > 2) {
        st |= kStSegOverflow;
        break;
      }
      int a0 = __ldg(S.cell_start + colbase + izw);
      int a1 = __ldg(S.cell_start + colbase + izw_end + 1);
      sm.seg_start[base + r] = a0;
      sm.seg_pref[base + r] = a1 - a0;
      sm.seg_shift[base + r] = (imx + 2) | ((imy + 2) << 4) | ((imz + 2) << 8);
      ++r;
      iz = run_end + 1;
    }
  }
  __syncthreads();
  // exclusive prefix over the slots: each thread owns a contiguous chunk
  int per = (nslot + kThreads - 1) / kThreads;
  int b = threadIdx.x * per, e = min(nslot, b + per);
  int local = 0;
  for (int i = b; i < e; ++i) local += sm.seg_pref[i];
  int excl;
  int tot = block_scan(local, excl, sm.red_i);
  int run = excl;
  for (int i = b; i < e; ++i) {
    int cnt = sm.seg_pref[i];
    sm.seg_pref[i] = run;
    run += cnt;
  }
  if (threadIdx.x == 0) {
    sm.seg_pref[nslot] = tot;
    sm.nslots = nslot;
  }
  __syncthreads();
}

__device__ __forceinline__ int find_slot(const int *pref, int n, int t) {
  // largest s in [0, n) with pref[s] <= t
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (pref[mid] <= t) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Scan the framework for position `pos` (ns sites).
// NS > 0: the site count is a compile-time constant (site loops unroll).
template <bool F32, int NS, bool TRIC, class PA>
__device__ __forceinline__ void scan_framework(const SysDev &S, EvalSmem<F32> &sm, int pos,
                                               int ns_rt, const SiteInfo *si, PA &acc, int &ov,
                                               int &sf, int &st) {
  const int ns = NS > 0 ? NS : ns_rt;
  int nslot = sm.nslots;
  const int t0 = 0, total = sm.seg_pref[nslot];  // this CTA's columns only
  if constexpr (!F32) {
    double e2 = 0.0, vdw = 0.0;
    for (int t = t0 + threadIdx.x; t < total; t += kThreads) {
      int s = find_slot(sm.seg_pref, nslot, t);
      int a = sm.seg_start[s] + (t - sm.seg_pref[s]);
      int sh = sm.seg_shift[s];
      double4 A = S.fw64[a];
      int tb = __ldg(S.fwtype + a);
      double ax = A.x + double((sh & 15) - 2) * S.box[0];
      double ay = A.y + double(((sh >> 4) & 15) - 2) * S.box[1];
      double az = A.z + double(((sh >> 8) & 15) - 2) * S.box[2];
      for (int k = 0; k < ns; ++k) {
        double dx = sm.p64[pos][k][0] - ax, dy = sm.p64[pos][k][1] - ay,
               dz = sm.p64[pos][k][2] - az;
        if (!S.use_cells) {  // parallelepiped: fractional minimum image
          const double *r = S.rcell, *c = S.cell;
          double fx = r[0] * dx + r[3] * dy + r[6] * dz;
          double fy = r[1] * dx + r[4] * dy + r[7] * dz;
          double fz = r[2] * dx + r[5] * dy + r[8] * dz;
          fx -= round(fx);
          fy -= round(fy);
          fz -= round(fz);
          dx = c[0] * fx + c[3] * fy + c[6] * fz;
          dy = c[1] * fx + c[4] * fy + c[7] * fz;
          dz = c[2] * fx + c[5] * fy + c[8] * fz;
        }
        double r2 = dx * dx + dy * dy + dz * dz;
        pair_term64(S, si[k], A.w, tb, 1, r2, e2, vdw, ov, sf, st);
      }
    }
    acc.e2fw.add(e2);
    acc.vdwfw.add(vdw);
  } else if (TRIC && !S.use_cells) {
    // parallelepiped cell: every atom of this CTA's share, minimum image
    // through the cell translation (mi_tric_df)
    float vdw = 0.0f;
    int cnt = 0;
    const int a0 = sm.seg_start[0];
    for (int t = t0 + threadIdx.x; t < total; t += kThreads) {
      const int a = a0 + t;
      const float4 H = __ldg(S.fwhi + a), Lo = __ldg(S.fwlo + a);
      const int tb = __ldg(S.fwtype + a);
      const float ah[3] = {H.x, H.y, H.z}, al[3] = {Lo.x, Lo.y, Lo.z};
#pragma unroll
      for (int k = 0; k < (NS > 0 ? NS : ns); ++k) {
        float dh[3], dl[3];
        mi_tric_df(S, sm.phi[pos][k], sm.plo[pos][k], ah, al, dh, dl);
        const float dx = dh[0] + dl[0], dy = dh[1] + dl[1], dz = dh[2] + dl[2];
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const bool near = vdw_is_near(S, si[k], tb, r2);
        pair_term32(S, si[k], H.w, Lo.w, tb, 1, r2, acc.e2fw, vdw, ov, sf, st, near);
        if (near) acc.vdwfw.add_df(vdw_near_df(S, si[k], tb, dh, dl, st));
      }
      if (++cnt == 8) {
        acc.vdwfw.add(vdw);
        vdw = 0.0f;
        cnt = 0;
      }
    }
    acc.vdwfw.add(vdw);
  } else {
    float vdw = 0.0f;
    int cnt = 0;
    const float *Lh = S.boxh, *Ll = S.boxl;
    for (int t = t0 + threadIdx.x; t < total; t += kThreads) {
      int s = find_slot(sm.seg_pref, nslot, t);
      int a = sm.seg_start[s] + (t - sm.seg_pref[s]);
      int sh = sm.seg_shift[s];
      float4 H = __ldg(S.fwhi + a);
      float4 Lo = __ldg(S.fwlo + a);
      int tb = __ldg(S.fwtype + a);
      float ah[3] = {H.x, H.y, H.z}, al[3] = {Lo.x, Lo.y, Lo.z};
      int im[3] = {(sh & 15) - 2, ((sh >> 4) & 15) - 2, ((sh >> 8) & 15) - 2};
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        if (im[d] != 0) {
          float h, e;
          two_sum_f(ah[d], float(im[d]) * Lh[d], h, e);
          ah[d] = h;
          al[d] = al[d] + (e + float(im[d]) * Ll[d]);
        }
      }
#pragma unroll
      for (int k = 0; k < (NS > 0 ? NS : ns); ++k) {
        float dx = (sm.phi[pos][k][0] - ah[0]) + (sm.plo[pos][k][0] - al[0]);
        float dy = (sm.phi[pos][k][1] - ah[1]) + (sm.plo[pos][k][1] - al[1]);
        float dz = (sm.phi[pos][k][2] - ah[2]) + (sm.plo[pos][k][2] - al[2]);
        float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const bool near = vdw_is_near(S, si[k], tb, r2);
        pair_term32(S, si[k], H.w, Lo.w, tb, 1, r2, acc.e2fw, vdw, ov, sf, st, near);
        if (near) {
          float dh[3], dl[3];
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            float e;
            two_sum_f(sm.phi[pos][k][d], -ah[d], dh[d], e);
            dl[d] = e + (sm.plo[pos][k][d] - al[d]);
          }
          acc.vdwfw.add_df(vdw_near_df(S, si[k], tb, dh, dl, st));
        }
      }
      if (++cnt == 8) {
        acc.vdwfw.add(vdw);
        vdw = 0.0f;
        cnt = 0;
      }
    }
    acc.vdwfw.add(vdw);
  }
}

// Guest-guest part: every molecule of every guest type except the moving
// one (the reference's ind exclusion, utility_pack.f:3736-3741).  Minimum
// image per site pair, as images() does for each list entry.
template <bool F32, int GN, int NS>
__device__ __forceinline__ void scan_guests(const SysDev &S, const ChainHdr &H,
                                            const ChainArrays &CA, int chain, EvalSmem<F32> &sm,
                                            int pos, int ns_rt, int self_g, int self_slot,
                                            float rmax_self, const SiteInfo *si,
                                            PosAcc<F32, GN> &acc, int &ov, int &sf, int &st) {
  const int ns = NS > 0 ? NS : ns_rt;
#pragma unroll
  for (int g2 = 0; g2 < GN; ++g2) {
    if (g2 >= S.ntpguest) break;
    const GuestType &G2 = S.g[g2];
    int n2 = H.nummols[g2];
    const int *ord = CA.ord + ((size_t)chain * kMaxG + g2) * CA.cap;
    float pre = (float)S.rcut + 2.0f * rmax_self + 2.0f * (float)G2.rmax + 0.01f;
    if constexpr (F32) {
      // parallelepiped cells only in the multi-type FP32 kernel
      const bool tric = GN > 1 && !S.use_cells;
      const float4 *gh = CA.ghi + ((size_t)chain * kMaxG + g2) * CA.cap * kMaxS;
      const float4 *gl = CA.glo + ((size_t)chain * kMaxG + g2) * CA.cap * kMaxS;
      float pre2 = pre * pre;
      int i0, i1;
      share_of(n2, sm.rank, sm.csize, i0, i1);
      for (int i = i0 + threadIdx.x; i < i1; i += kThreads) {
        int slot = ord[i];
        if ((unsigned)slot >= (unsigned)CA.cap) {  // a damaged order list: skipped, reported
          st |= kStIndex;
          continue;
        }
        if (g2 == self_g && slot == self_slot) continue;
        float4 q0 = gh[(size_t)slot * kMaxS];
        float dx = sm.phi[pos][0][0] - q0.x, dy = sm.phi[pos][0][1] - q0.y,
              dz = sm.phi[pos][0][2] - q0.z;
        if (!tric) {
          dx -= S.boxh[0] * rint_image(dx * S.rboxf[0]);
          dy -= S.boxh[1] * rint_image(dy * S.rboxf[1]);
          dz -= S.boxh[2] * rint_image(dz * S.rboxf[2]);
          if (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) > pre2) continue;
        } else if (tric_r2_f32(S, dx, dy, dz) > pre2) {
          continue;
        }
        float vdw = 0.f;
        for (int b = 0; b < G2.ns; ++b) {
          float4 qh = gh[(size_t)slot * kMaxS + b];
          float4 ql = gl[(size_t)slot * kMaxS + b];
          int tb = G2.type[b];
#pragma unroll
          for (int k = 0; k < (NS > 0 ? NS : ns); ++k) {
            float dh[3], dl[3], ex, ey, ez;
            if (!tric) {
              ex = mi_diff32(sm.phi[pos][k][0], sm.plo[pos][k][0], qh.x, ql.x, S.boxh[0],
                             S.boxl[0], S.rboxf[0]);
              ey = mi_diff32(sm.phi[pos][k][1], sm.plo[pos][k][1], qh.y, ql.y, S.boxh[1],
                             S.boxl[1], S.rboxf[1]);
              ez = mi_diff32(sm.phi[pos][k][2], sm.plo[pos][k][2], qh.z, ql.z, S.boxh[2],
                             S.boxl[2], S.rboxf[2]);
            } else {  // parallelepiped cell
              const float qa[3] = {qh.x, qh.y, qh.z}, qb[3] = {ql.x, ql.y, ql.z};
              mi_tric_df(S, sm.phi[pos][k], sm.plo[pos][k], qa, qb, dh, dl);
              ex = dh[0] + dl[0];
              ey = dh[1] + dl[1];
              ez = dh[2] + dl[2];
            }
            float r2 = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
            const bool near = vdw_is_near(S, si[k], tb, r2);
            pair_term32(S, si[k], qh.w, ql.w, tb, G2.frz[b], r2, acc.e2g[g2], vdw, ov, sf, st,
                        near);
            if (near) {
              if (!tric) {
                mi_diff_df(sm.phi[pos][k][0], sm.plo[pos][k][0], qh.x, ql.x, S.boxh[0],
                           S.boxl[0], S.rboxf[0], dh[0], dl[0]);
                mi_diff_df(sm.phi[pos][k][1], sm.plo[pos][k][1], qh.y, ql.y, S.boxh[1],
                           S.boxl[1], S.rboxf[1], dh[1], dl[1]);
                mi_diff_df(sm.phi[pos][k][2], sm.plo[pos][k][2], qh.z, ql.z, S.boxh[2],
                           S.boxl[2], S.rboxf[2], dh[2], dl[2]);
              }
              acc.vdwg[g2].add_df(vdw_near_df(S, si[k], tb, dh, dl, st));
            }
          }
        }
        acc.vdwg[g2].add(vdw);
      }
    } else {
      double pre2 = (double)pre * (double)pre;
      double e2 = 0.0, vdw = 0.0;
      int i0, i1;
      share_of(n2, sm.rank, sm.csize, i0, i1);
      for (int i = i0 + threadIdx.x; i < i1; i += kThreads) {
        int slot = ord[i];
        if ((unsigned)slot >= (unsigned)CA.cap) {  // a damaged order list: skipped, reported
          st |= kStIndex;
          continue;
        }
        if (g2 == self_g && slot == self_slot) continue;
        size_t base = (((size_t)chain * kMaxG + g2) * CA.cap + slot) * kMaxS;
        const double *q0 = CA.gpos + base * 3;
        if (S.use_cells) {  // prefilter on site 0 - site 0
          double dx = sm.p64[pos][0][0] - q0[0], dy = sm.p64[pos][0][1] - q0[1],
                 dz = sm.p64[pos][0][2] - q0[2];
          dx -= S.box[0] * round(S.rbox[0] * dx);
          dy -= S.box[1] * round(S.rbox[1] * dy);
          dz -= S.box[2] * round(S.rbox[2] * dz);
          if (dx * dx + dy * dy + dz * dz > pre2) continue;
        }
        for (int b = 0; b < G2.ns; ++b) {
          const double *qb = CA.gpos + (base + b) * 3;
          double qq = G2.q[b];
          int tb = G2.type[b];
          for (int k = 0; k < ns; ++k) {
            double ddx = sm.p64[pos][k][0] - qb[0], ddy = sm.p64[pos][k][1] - qb[1],
                   ddz = sm.p64[pos][k][2] - qb[2];
            if (S.use_cells) {
              ddx -= S.box[0] * round(S.rbox[0] * ddx);
              ddy -= S.box[1] * round(S.rbox[1] * ddy);
              ddz -= S.box[2] * round(S.rbox[2] * ddz);
            } else {
              const double *r = S.rcell, *c = S.cell;
              double fx = r[0] * ddx + r[3] * ddy + r[6] * ddz;
              double fy = r[1] * ddx + r[4] * ddy + r[7] * ddz;
              double fz = r[2] * ddx + r[5] * ddy + r[8] * ddz;
              fx -= round(fx);
              fy -= round(fy);
              fz -= round(fz);
              ddx = c[0] * fx + c[3] * fy + c[6] * fz;
              ddy = c[1] * fx + c[4] * fy + c[7] * fz;
              ddz = c[2] * fx + c[5] * fy + c[8] * fz;
            }
            double r2 = ddx * ddx + ddy * ddy + ddz * ddz;
            pair_term64(S, si[k], qq, tb, G2.frz[b], r2, e2, vdw, ov, sf, st);
          }
        }
      }
      acc.e2g[g2].add(e2);
      acc.vdwg[g2].add(vdw);
    }
  }
}

// ----------------------------------------------------------------- k-space
// Power tables e^{i 2 pi j s_d} for npos positions of ns sites
// (the first harmonics and recurrences of ewald.f:108-147, evaluated
// directly for each power j).  FP64 path: sincospi of the reduced phase.
// FP32 path: the fractional coordinate is split into a float hi/lo pair
// and j*s is reduced exactly with an FMA before sincospif.
template <bool F32, bool TRIC>
__device__ void build_powers(const SysDev &S, EvalSmem<F32> &sm, int npos, int ns) {
  int k1 = S.kmax[0], k2 = S.kmax[1], k3 = S.kmax[2];
  if constexpr (F32) {
    // fractional coordinate x / L of the hi/lo position as a hi/lo pair
    // (orthorhombic cells), reduced by whole cells: e^{i 2 pi j f} only
    // needs f modulo 1
    int nf = npos * ns * 3;
    if (threadIdx.x < nf) {
      int pos = threadIdx.x / (ns * 3), rem = threadIdx.x % (ns * 3), s = rem / 3, d = rem % 3;
      float fh, fe;
      if (!TRIC || S.use_cells) {
        const float xh = sm.phi[pos][s][d], xl = sm.plo[pos][s][d];
        const float rh = S.rboxf[d], rl = S.rboxf_lo[d];
        fh = xh * rh;
        fe = fmaf(xh, rh, -fh) + fmaf(xh, rl, xl * rh);
      } else {  // parallelepiped: rcell row d times the position, double-float
        fh = 0.f;
        fe = 0.f;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const float xh = sm.phi[pos][s][j], xl = sm.plo[pos][s][j];
          const float rh = S.rcellh[d + 3 * j], rl = S.rcelll[d + 3 * j];
          const float p = xh * rh;
          const float pe = fmaf(xh, rh, -p) + fmaf(xh, rl, xl * rh);
          float t, e;
          two_sum_f(fh, p, t, e);
          fh = t;
          fe += e + pe;
        }
      }
      float s0, e0, hi, lo;
      two_sum_f(fh, -floorf(fh), s0, e0);
      two_sum_f(s0, e0 + fe, hi, lo);
      sm.fhi[pos][s][d] = hi;
      sm.flo[pos][s][d] = lo;
    }
    __syncthreads();
  }
  int per = k1 + k2 + k3 + 3;
  int total = npos * ns * per;
  for (int t = threadIdx.x; t < total; t += kThreads) {
    int pos = t / (ns * per);
    int rem = t % (ns * per);
    int s = rem / per;
    int j = rem % per;
    int d = 0;
    if (j > k1) {
      j -= k1 + 1;
      d = 1;
      if (j > k2) {
        j -= k2 + 1;
        d = 2;
      }
    }
    if constexpr (!F32) {
      const double *p = sm.p64[pos][s];
      const double *r = S.rcell;
      double f = r[d] * p[0] + r[3 + d] * p[1] + r[6 + d] * p[2];
      double x = double(j) * f;
      x -= rint(x);
      double sn, cs;
      sincospi(2.0 * x, &sn, &cs);
      sm.pw64[pos][s][d][j] = make_double2(cs, sn);
    } else {
      float fj = (float)j;
      float ph = fj * sm.fhi[pos][s][d];
      float pe = fmaf(fj, sm.fhi[pos][s][d], -ph);  // exact product error
      float x = (ph - rintf(ph)) + fmaf(fj, sm.flo[pos][s][d], pe);
      float sn, cs;
      sincospif(2.0f * x, &sn, &cs);
      sm.pw32[pos][s][d][j] = make_float2(cs, sn);
    }
  }
  if constexpr (F32) {
    // (l, m) products, so the k loop needs one complex product per site
    const int w = 2 * k2 + 1, nlm = (k1 + 1) * w;
    if (sm.tabpos * ns * nlm <= kPlmMax) {
      __syncthreads();
      for (int e = threadIdx.x; e < nlm; e += kThreads) {
        const int l = e / w, mm = e - l * w - k2, am = abs(mm);
        for (int p = 0; p < npos; ++p)
          for (int s = 0; s < ns; ++s) {
            const float2 X = sm.pw32[p][s][0][l];
            float2 Y = sm.pw32[p][s][1][am];
            if (mm < 0) Y.y = -Y.y;
            sm.plm[(p * ns + s) * nlm + e] = make_float2(X.x * Y.x - X.y * Y.y, X.y * Y.x + X.x * Y.y);
          }
      }
    }
  }
}

template <class T2>
__device__ __forceinline__ T2 cmul(T2 a, T2 b) {
  T2 r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.y * b.x + a.x * b.y;
  return r;
}

}  // namespace fmcdev

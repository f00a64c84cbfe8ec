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
//     its energy against S(k) and the per-molecule-type mixing terms.
#pragma once

#include "device_core.cuh"

namespace fmcdev {

template <bool F32>
struct EvalSmem {
  double p64[2][kMaxS][3];
  float phi[2][kMaxS][3];
  float plo[2][kMaxS][3];
  // power tables e^{i 2 pi j s_d}: [pos][site][axis][j]
  double2 pw64[F32 ? 1 : 2][F32 ? 1 : kMaxS][3][F32 ? 1 : kMaxKm];
  float2 pw32[F32 ? 2 : 1][F32 ? kMaxS : 1][3][F32 ? kMaxKm : 1];
  int seg_start[kMaxSeg];
  int seg_pref[kMaxSeg + 1];
  int seg_shift[kMaxSeg];
  int nslots;
  int red_i[kWarps + 1];
  double red[kWarps * 48 + 48];
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
  int type;
};

// One site-atom pair.  Adds the erfc and van der Waals terms when r < rc,
// sets the overlap and surface flags like surface_check.
template <bool F32>
__device__ __forceinline__ void pair_term64(const SysDev &S, const SiteInfo &si,
                                            double qb, int tb, int frozen_b,
                                            double r2, double &e2, double &vdw,
                                            int &ov, int &sf, int &st) {
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

__device__ __forceinline__ void pair_term32(const SysDev &S, const SiteInfo &si,
                                            float chgprd, int tb, int frozen_b,
                                            float r2, float &e2, float &vdw,
                                            int &ov, int &sf, int &st) {
  int pi = si.type * (S.ntpatm + 1) + tb;
  if (r2 < (float)S.overlap_sq) ov = 1;
  if (frozen_b && r2 < (float)__ldg(S.sig2 + pi)) sf = 1;
  if (r2 < (float)S.rc2) {
    float r = sqrtf(r2);
    if (fabsf(chgprd) > 1.0e-10f)
      e2 = fmaf(interp32(S.ercq, r, (float)S.rdrewd, S.mxegrd, st), chgprd, e2);
    int k = __ldg(S.pairtab + pi);
    if (k >= 0) vdw += interp32(S.vvvq + (size_t)k * S.tabstride, r, (float)S.rdlrpot, S.mxegrd, st);
  }
}

// Error-free sum a + b = s + e.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// ---------------------------------------------------- framework neighbours
// Build the list of framework atom segments (runs of cells along z in one
// column and one periodic image) that cover the sphere of radius R around
// c.  Slots with zero atoms are allowed; seg_pref is the prefix over slots.
template <bool F32>
__device__ void build_segments(const SysDev &S, EvalSmem<F32> &sm, const double *c,
                               double R, int &st) {
  if (!S.use_cells) {
    if (threadIdx.x == 0) {
      sm.seg_start[0] = 0;
      sm.seg_shift[0] = (2) | (2 << 4) | (2 << 8);
      sm.seg_pref[0] = 0;
      sm.seg_pref[1] = S.nfw;
      sm.nslots = 1;
    }
    __syncthreads();
    return;
  }
  int ix0 = (int)floor((c[0] - R) / S.csz[0]), ix1 = (int)floor((c[0] + R) / S.csz[0]);
  int iy0 = (int)floor((c[1] - R) / S.csz[1]), iy1 = (int)floor((c[1] + R) / S.csz[1]);
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
  double R2 = R * R;
  for (int col = threadIdx.x; col < ncol; col += kThreads) {
    int ix = ix0 + col / ny, iy = iy0 + col % ny;
    double xlo = ix * S.csz[0], xhi = xlo + S.csz[0];
    double ylo = iy * S.csz[1], yhi = ylo + S.csz[1];
    double dx = fmax(0.0, fmax(xlo - c[0], c[0] - xhi));
    double dy = fmax(0.0, fmax(ylo - c[1], c[1] - yhi));
    double d2 = dx * dx + dy * dy;
    int base = col * kRuns;
    for (int r = 0; r < kRuns; ++r) {
      sm.seg_start[base + r] = 0;
      sm.seg_shift[base + r] = 0;
      sm.seg_pref[base + r] = 0;  // count for now
    }
    if (d2 > R2) continue;
    double hz = sqrt(R2 - d2);
    int iz0 = (int)floor((c[2] - hz) / S.csz[2]), iz1 = (int)floor((c[2] + hz) / S.csz[2]);
    int imx = (ix >= 0) ? ix / S.nc[0] : -((-ix + S.nc[0] - 1) / S.nc[0]);
    int imy = (iy >= 0) ? iy / S.nc[1] : -((-iy + S.nc[1] - 1) / S.nc[1]);
    int ixw = ix - imx * S.nc[0], iyw = iy - imy * S.nc[1];
    int colbase = (ixw * S.nc[1] + iyw) * S.nc[2];
    int r = 0;
    int iz = iz0;
    while (iz <= iz1) {
      int imz = (iz >= 0) ? iz / S.nc[2] : -((-iz + S.nc[2] - 1) / S.nc[2]);
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
  // largest s in [0, n) with pref[s] <= t and pref[s+1] > t
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (pref[mid] <= t) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Scan the framework for position `pos` (ns sites) and accumulate into acc.
template <bool F32>
__device__ void scan_framework(const SysDev &S, EvalSmem<F32> &sm, int pos, int ns,
                               const SiteInfo *si, Acc &acc, int &ov, int &sf,
                               int &st) {
  int nslot = sm.nslots;
  int total = sm.seg_pref[nslot];
  if constexpr (!F32) {
    double e2 = 0.0, vdw = 0.0;
    for (int t = threadIdx.x; t < total; t += kThreads) {
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
        pair_term64<false>(S, si[k], A.w, tb, 1, r2, e2, vdw, ov, sf, st);
      }
    }
    acc.e2_fw += e2;
    acc.vdw_fw += vdw;
  } else {
    float e2 = 0.0f, vdw = 0.0f;
    double e2d = 0.0, vdwd = 0.0;
    int cnt = 0;
    const float Lh[3] = {(float)S.box[0], (float)S.box[1], (float)S.box[2]};
    const float Ll[3] = {(float)(S.box[0] - (double)Lh[0]), (float)(S.box[1] - (double)Lh[1]),
                         (float)(S.box[2] - (double)Lh[2])};
    for (int t = threadIdx.x; t < total; t += kThreads) {
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
          two_sum(ah[d], float(im[d]) * Lh[d], h, e);
          ah[d] = h;
          al[d] = al[d] + (e + float(im[d]) * Ll[d]);
        }
      }
      for (int k = 0; k < ns; ++k) {
        float dx = (sm.phi[pos][k][0] - ah[0]) + (sm.plo[pos][k][0] - al[0]);
        float dy = (sm.phi[pos][k][1] - ah[1]) + (sm.plo[pos][k][1] - al[1]);
        float dz = (sm.phi[pos][k][2] - ah[2]) + (sm.plo[pos][k][2] - al[2]);
        float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        float chgprd = (float)si[k].chgea * H.w;
        pair_term32(S, si[k], chgprd, tb, 1, r2, e2, vdw, ov, sf, st);
      }
      if (++cnt == 8) {
        e2d += e2;
        vdwd += vdw;
        e2 = vdw = 0.0f;
        cnt = 0;
      }
    }
    acc.e2_fw += e2d + (double)e2;
    acc.vdw_fw += vdwd + (double)vdw;
  }
}

// Guest-guest part: every molecule of every guest type except the moving
// one (the reference's ind exclusion, utility_pack.f:3736-3741).
template <bool F32>
__device__ void scan_guests(const SysDev &S, const ChainHdr &H, const ChainArrays &CA,
                            int chain, EvalSmem<F32> &sm, int pos, int ns, int self_g,
                            int self_slot, double rmax_self, const SiteInfo *si,
                            Acc &acc, int &ov, int &sf, int &st) {
  for (int g2 = 0; g2 < S.ntpguest; ++g2) {
    const GuestType &G2 = S.g[g2];
    int n2 = H.nummols[g2];
    const int *ord = CA.ord + ((size_t)chain * kMaxG + g2) * CA.cap;
    double pre = S.rcut + 2.0 * rmax_self + 2.0 * G2.rmax + 0.01;
    double pre2 = pre * pre;
    double e2 = 0.0, vdw = 0.0;
    for (int i = threadIdx.x; i < n2; i += kThreads) {
      int slot = ord[i];
      if (g2 == self_g && slot == self_slot) continue;
      size_t base = (((size_t)chain * kMaxG + g2) * CA.cap + slot) * kMaxS;
      // prefilter on site 0 - site 0 (minimum image)
      const double *q0 = CA.gpos + base * 3;
      double dx = sm.p64[pos][0][0] - q0[0], dy = sm.p64[pos][0][1] - q0[1],
             dz = sm.p64[pos][0][2] - q0[2];
      if (S.use_cells) {
        dx -= S.box[0] * round(dx / S.box[0]);
        dy -= S.box[1] * round(dy / S.box[1]);
        dz -= S.box[2] * round(dz / S.box[2]);
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
            ddx -= S.box[0] * round(ddx / S.box[0]);
            ddy -= S.box[1] * round(ddy / S.box[1]);
            ddz -= S.box[2] * round(ddz / S.box[2]);
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
          if constexpr (!F32) {
            pair_term64<false>(S, si[k], qq, tb, G2.frz[b], r2, e2, vdw, ov, sf, st);
          } else {
            float fe2 = 0.0f, fv = 0.0f;
            pair_term32(S, si[k], (float)(si[k].chgea * qq), tb, G2.frz[b], (float)r2,
                        fe2, fv, ov, sf, st);
            e2 += fe2;
            vdw += fv;
          }
        }
      }
    }
    acc.e2_g[g2] += e2;
    acc.vdw_g[g2] += vdw;
  }
}

// ----------------------------------------------------------------- k-space
// Power tables for npos positions of ns sites.
template <bool F32>
__device__ void build_powers(const SysDev &S, EvalSmem<F32> &sm, int npos, int ns) {
  int k1 = S.kmax[0], k2 = S.kmax[1], k3 = S.kmax[2];
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
    const double *p = sm.p64[pos][s];
    const double *r = S.rcell;
    double f = r[d] * p[0] + r[3 + d] * p[1] + r[6 + d] * p[2];
    double x = double(j) * f;
    x -= rint(x);
    if constexpr (!F32) {
      double sn, cs;
      sincospi(2.0 * x, &sn, &cs);
      sm.pw64[pos][s][d][j] = make_double2(cs, sn);
    } else {
      float sn, cs;
      sincospif((float)(2.0 * x), &sn, &cs);
      sm.pw32[pos][s][d][j] = make_float2(cs, sn);
    }
  }
}

// e^{i k.r} for one site from the power tables, with the reference's sign
// conventions for negative m and n (ewald.f:191-251).
template <class T2>
__device__ __forceinline__ T2 cmul(T2 a, T2 b) {
  T2 r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.y * b.x + a.x * b.y;
  return r;
}

}  // namespace fmcdev

// engine.cuh -- the GCMC move loop of one chain on one CTA.
//
// Phases of one main-loop iteration (gcmc.f:704-1164):
//   propose  (thread 0)  guest and move choice, adaptive step sizes,
//                        trial geometry from the MZT generator;
//   evaluate (all)       overlap pre-check, pair scans, k-space, fixed-order
//                        reductions, estep and delE as the reference forms
//                        them (mc_moves.f:150-484, gcmc.f:2816-2901);
//   decide   (thread 0)  energy_eval (utility_pack.f:3637-3693);
//   commit   (all)       accept_move (mc_moves.f:485-621): S(k), molecule
//                        order, coordinates, counters;
//   stats    (thread 0)  production averages and windows (gcmc.f:1050-1128).
#pragma once

#include "device_eval.cuh"

namespace fmcdev {

struct LogRec {  // mirrors fmc_move_log
  int move, iguest, choice, overlap, accepted, nmols_after;
  double estep, rande;
  double newxyz[9];
};

template <bool F32>
struct BlockShared {
  SysDev S;
  ChainHdr H;
  MoveCtx mc;
  EvalSmem<F32> ev;
  SiteInfo si[kMaxS];
  int flags[4];
};

__device__ __forceinline__ size_t gslot_base(const ChainArrays &CA, int chain, int g, int slot) {
  return (((size_t)chain * kMaxG + g) * CA.cap + slot) * kMaxS;
}

// ------------------------------------------------- per-guest LJ tail delta
// gstlrcorrect (vdw_terms.f:686-776) from the chain's type counters.
__device__ void gst_lrc(const SysDev &S, const ChainHdr &H, int g, bool lexisting,
                        double &delrc, double *delrc_mol) {
  const GuestType &G = S.g[g];
  int mol = G.mol;
  double twopi = 2.0 * kPi;
  int ntg[kMaxT + 1], nfg[kMaxT + 1];
  for (int a = 0; a <= S.ntpatm; ++a) ntg[a] = nfg[a] = 0;
  for (int s = 0; s < G.ns; ++s) {
    ntg[G.type[s]]++;
    if (G.frz[s]) nfg[G.type[s]]++;
  }
  delrc = 0.0;
  for (int m = 0; m <= S.maxmls; ++m) delrc_mol[m] = 0.0;
  int iv = 0;
  double v2 = S.volm * S.volm;
  for (int i = 1; i <= S.ntpatm; ++i)
    for (int j = 1; j <= i; ++j) {
      ++iv;
      double eadd = S.steadd[iv];
      double na = ntg[i], nb = ntg[j], fa = nfg[i], fb = nfg[j];
      double den = na * double(H.numtyp[j]) + nb * double(H.numtyp[i]) -
                   fa * double(H.numfrz[j]) - fb * double(H.numfrz[i]);
      if (lexisting) den = -1.0 * den;
      den = den + (na * nb - fa * fb);
      delrc = delrc + S.volm * twopi * den / v2 * eadd;
      for (int jt = 1; jt <= S.maxmls; ++jt) {
        double nc = H.numtyp_mol[jt][j], nd = H.numtyp_mol[jt][i];
        double fc = H.numfrz_mol[jt][j], fd = H.numfrz_mol[jt][i];
        double sic = na * nc + nb * nd - fa * fc - fb * fd, self = 0.0;
        if (jt == mol) {
          self = na * nb - fa * fb;
          if (lexisting) sic = -1.0 * sic;
        }
        delrc_mol[jt] += S.volm * eadd * (twopi * (sic + self) / v2);
      }
    }
}

// energy_eval (utility_pack.f:3637-3693)
__device__ bool energy_eval(const SysDev &S, const ChainHdr &H, int g, double eng,
                            double rande, int kind) {
  double ipress = H.fuga[g];
  int ing = H.nummols[g];
  double beta = S.beta, test = 0.0;
  if (-beta * eng > 700.0) test = exp(700.0);
  else if (beta * eng > 700.0) test = exp(-700.0);
  else if (kind >= 3) test = exp(-1.0 * beta * eng);
  else if (kind == 1)
    test = S.statvolm * ipress / ((double(ing) + 1.0) * kBoltz * S.temp) * exp(-1.0 * beta * eng);
  else if (kind == 2) {
    if (fabs(ipress) < 1.0e-7) test = 1.0;
    else test = double(ing) * kBoltz * S.temp / (S.statvolm * ipress) * exp(-1.0 * beta * eng);
  }
  return rande < test;
}

// ----------------------------------------------------------------- propose
// Thread 0: one iteration's draws (gcmc.f:806-900, 1693-1870).  Returns
// false if the chain has nothing to do this step.
template <bool F32>
__device__ void propose(BlockShared<F32> &B, const ChainArrays &CA, int chain) {
  SysDev &S = B.S;
  ChainHdr &H = B.H;
  MoveCtx &mc = B.mc;
  H.gcmccount++;
  if (H.gcmccount % S.minchk == 0)
    if (!H.production && S.eqsteps > 0 && H.gcmccount >= S.eqsteps) H.production = 1;
  int g = 0;
  if (S.ntpguest > 1) g = (int)floor(duni_next(H) * S.ntpguest);
  const GuestType &G = S.g[g];
  int nmols = H.nummols[g];
  double randmov = duni_next(H);
  int kind;
  if (randmov < G.mcinsf) kind = 1;
  else if (randmov < G.mcdelf) kind = 2;
  else if (randmov < G.mcdisf) kind = 3;
  else if (randmov < G.mcjmpf) kind = 3;  // not reachable: refused at set-up
  else if (randmov < G.mcswpf) kind = 3;
  else if (randmov < G.mctraf) kind = 4;
  else if (randmov < G.mcrotf) kind = 5;
  else kind = 3;
  // adaptive step sizes (gcmc.f:859-900)
  if (nmols >= 1 && H.disp_count[g] >= 1) {
    double ratio = double(H.accept_disp[g]) / double(H.disp_count[g]);
    if (H.disp_count[g] % 100 == 0) {
      if (ratio > G.disp_ratio) H.delrdisp[g] *= 1.05;
      else if (H.delrdisp[g] > kDelrMin) H.delrdisp[g] *= 0.95;
    } else if (H.disp_count[g] % 50 == 0) {
      if (ratio > G.disp_ratio) H.rotangle *= 1.05;
      else if (H.rotangle > kMinAngle) H.rotangle *= 0.95;
    }
  }
  if (nmols >= 1 && H.tran_count[g] >= 1 && H.tran_count[g] % 100 == 0) {
    double ratio = double(H.accept_tran[g]) / double(H.tran_count[g]);
    if (ratio > G.tran_ratio) H.tran_delr[g] *= 1.05;
    else if (H.tran_delr[g] > kDelrMin) H.tran_delr[g] *= 0.95;
  }
  if (nmols >= 1 && H.rota_count[g] >= 1 && H.rota_count[g] % 100 == 0) {
    double ratio = double(H.accept_rota[g]) / double(H.rota_count[g]);
    if (ratio > G.rota_ratio) H.rota_rotangle *= 1.05;
    else if (H.rota_rotangle > kMinAngle) H.rota_rotangle *= 0.95;
  }
  if (nmols == 0) kind = 1;
  mc.kind = kind;
  mc.g = g;
  mc.ns = G.ns;
  mc.rande = -1.0;
  mc.estep = 0.0;
  mc.overlap = 0;
  mc.accepted = 0;
  mc.surf_new = mc.surf_old = 0;
  mc.npos = 1;
  mc.choice = 0;
  mc.slot = -1;
  if (kind == 1) {
    H.ins_count[g]++;
    // random_ins (utility_pack.f:3220-3331)
    double ra = duni_next(H), rb = duni_next(H), rc = duni_next(H);
    double r1 = duni_next(H), r2 = duni_next(H), r3 = duni_next(H), r4 = duni_next(H);
    double cc[3];
    cartesian(S, ra, rb, rc, cc);
    for (int s = 0; s < G.ns; ++s)
      for (int d = 0; d < 3; ++d) mc.pos[0][s][d] = G.tmpl[s][d];
    double q[4], zero[3] = {0.0, 0.0, 0.0};
    quaternion(r1, r2, r3, r4, 2.0 * kPi, q);
    rotate_sites(mc.pos[0], G.ns, zero, q[0], q[1], q[2], q[3]);
    for (int s = 0; s < G.ns; ++s)
      for (int d = 0; d < 3; ++d) mc.pos[0][s][d] += cc[d];
  } else if (kind == 2) {
    H.del_count[g]++;
    int choice = (int)floor(duni_next(H) * nmols) + 1;
    mc.choice = choice;
  } else {
    double a = 0, b = 0, c = 0, q[4] = {0, 0, 0, 0};
    auto disp = [&](double dd) {
      a = duni_next(H);
      b = duni_next(H);
      c = duni_next(H);
      double h = dd * 0.5;
      a = (2.0 * a - 1.0) * h;
      b = (2.0 * b - 1.0) * h;
      c = (2.0 * c - 1.0) * h;
    };
    auto rot = [&](double ang) {
      double r1 = duni_next(H), r2 = duni_next(H), r3 = duni_next(H), r4 = duni_next(H);
      quaternion(r1, r2, r3, r4, ang, q);
    };
    if (kind == 4) {
      H.tran_count[g]++;
      disp(H.tran_delr[g]);
    } else if (kind == 5) {
      H.rota_count[g]++;
      rot(H.rota_rotangle);
    } else {
      H.disp_count[g]++;
      disp(H.delrdisp[g]);
      rot(H.rotangle);
    }
    int choice = (int)floor(duni_next(H) * nmols) + 1;
    mc.choice = choice;
    mc.pos[1][0][0] = a;  // stash shift and quaternion for geometry()
    mc.pos[1][0][1] = b;
    mc.pos[1][0][2] = c;
    mc.pos[1][1][0] = q[0];
    mc.pos[1][1][1] = q[1];
    mc.pos[1][1][2] = q[2];
    mc.pos[1][2][0] = q[3];
  }
}

// Thread 0: molecule lookup and trial geometry for delete / displace
// (get_guest utility_pack.f:3776-3807, translate + rotation gcmc.f:2873-2876).
template <bool F32>
__device__ void geometry(BlockShared<F32> &B, const ChainArrays &CA, int chain) {
  SysDev &S = B.S;
  ChainHdr &H = B.H;
  MoveCtx &mc = B.mc;
  const GuestType &G = S.g[mc.g];
  if (mc.kind == 1) return;
  int nm = H.nummols[mc.g];
  if (mc.choice < 1 || mc.choice > nm) {
    H.status |= kStBadChoice;
    mc.kind = 0;
    return;
  }
  int slot = CA.ord[((size_t)chain * kMaxG + mc.g) * CA.cap + (mc.choice - 1)];
  mc.slot = slot;
  const double *src = CA.gpos + gslot_base(CA, chain, mc.g, slot) * 3;
  if (mc.kind == 2) {
    for (int s = 0; s < G.ns; ++s)
      for (int d = 0; d < 3; ++d) mc.pos[0][s][d] = src[3 * s + d];
    return;
  }
  double a = mc.pos[1][0][0], b = mc.pos[1][0][1], c = mc.pos[1][0][2];
  double q1 = mc.pos[1][1][0], q2 = mc.pos[1][1][1], q3 = mc.pos[1][1][2],
         q4 = mc.pos[1][2][0];
  for (int s = 0; s < G.ns; ++s)
    for (int d = 0; d < 3; ++d) {
      mc.pos[1][s][d] = src[3 * s + d];
      mc.pos[0][s][d] = src[3 * s + d];
    }
  translate_sites(S, G, mc.pos[0], a, b, c);
  double cm[3];
  centre_of_mass(G, mc.pos[0], cm);
  rotate_sites(mc.pos[0], G.ns, cm, q1, q2, q3, q4);
  mc.npos = 2;
}

// ------------------------------------------------------------- overlap test
// Any framework or guest site within the overlap distance of any site of
// position 0 (the pre-check that lets an insertion or displacement exit
// before the full sums, as insertion / guest_energy do, mc_moves.f:221-225).
template <bool F32>
__device__ int overlap_check(BlockShared<F32> &B, const ChainArrays &CA, int chain) {
  const SysDev &S = B.S;
  const MoveCtx &mc = B.mc;
  int ns = mc.ns;
  int hit = 0;
  if (S.use_cells) {
    int nrad = 1;
    double ov = sqrt(S.overlap_sq);
    while (nrad * fmin(S.csz[0], fmin(S.csz[1], S.csz[2])) < ov && nrad < 4) ++nrad;
    int span = 2 * nrad + 1;
    int per_site = span * span * span;
    for (int t = threadIdx.x; t < ns * per_site && !hit; t += kThreads) {
      int s = t / per_site, c = t % per_site;
      int ox = c / (span * span) - nrad, oy = (c / span) % span - nrad, oz = c % span - nrad;
      const double *p = mc.pos[0][s];
      int ix = (int)floor(p[0] / S.csz[0]) + ox, iy = (int)floor(p[1] / S.csz[1]) + oy,
          iz = (int)floor(p[2] / S.csz[2]) + oz;
      int imx = (ix >= 0) ? ix / S.nc[0] : -((-ix + S.nc[0] - 1) / S.nc[0]);
      int imy = (iy >= 0) ? iy / S.nc[1] : -((-iy + S.nc[1] - 1) / S.nc[1]);
      int imz = (iz >= 0) ? iz / S.nc[2] : -((-iz + S.nc[2] - 1) / S.nc[2]);
      int cell = ((ix - imx * S.nc[0]) * S.nc[1] + (iy - imy * S.nc[1])) * S.nc[2] +
                 (iz - imz * S.nc[2]);
      int a0 = __ldg(S.cell_start + cell), a1 = __ldg(S.cell_start + cell + 1);
      for (int a = a0; a < a1; ++a) {
        double4 A = S.fw64[a];
        double dx = p[0] - (A.x + imx * S.box[0]), dy = p[1] - (A.y + imy * S.box[1]),
               dz = p[2] - (A.z + imz * S.box[2]);
        if (dx * dx + dy * dy + dz * dz < S.overlap_sq) hit = 1;
      }
    }
  } else {
    for (int t = threadIdx.x; t < ns * S.nfw && !hit; t += kThreads) {
      int s = t / S.nfw, a = t % S.nfw;
      const double *p = mc.pos[0][s];
      double4 A = S.fw64[a];
      double dx = p[0] - A.x, dy = p[1] - A.y, dz = p[2] - A.z;
      const double *r = S.rcell, *c = S.cell;
      double fx = r[0] * dx + r[3] * dy + r[6] * dz, fy = r[1] * dx + r[4] * dy + r[7] * dz,
             fz = r[2] * dx + r[5] * dy + r[8] * dz;
      fx -= round(fx);
      fy -= round(fy);
      fz -= round(fz);
      dx = c[0] * fx + c[3] * fy + c[6] * fz;
      dy = c[1] * fx + c[4] * fy + c[7] * fz;
      dz = c[2] * fx + c[5] * fy + c[8] * fz;
      if (dx * dx + dy * dy + dz * dz < S.overlap_sq) hit = 1;
    }
  }
  // guests
  const GuestType &G = S.g[mc.g];
  for (int g2 = 0; g2 < S.ntpguest && !hit; ++g2) {
    const GuestType &G2 = S.g[g2];
    int n2 = B.H.nummols[g2];
    const int *ord = CA.ord + ((size_t)chain * kMaxG + g2) * CA.cap;
    double pre = sqrt(S.overlap_sq) + 2.0 * G.rmax + 2.0 * G2.rmax + 0.01;
    for (int i = threadIdx.x; i < n2 && !hit; i += kThreads) {
      int slot = ord[i];
      if (g2 == mc.g && slot == mc.slot) continue;
      const double *q = CA.gpos + gslot_base(CA, chain, g2, slot) * 3;
      double dx = mc.pos[0][0][0] - q[0], dy = mc.pos[0][0][1] - q[1], dz = mc.pos[0][0][2] - q[2];
      if (S.use_cells) {
        dx -= S.box[0] * round(dx / S.box[0]);
        dy -= S.box[1] * round(dy / S.box[1]);
        dz -= S.box[2] * round(dz / S.box[2]);
        if (dx * dx + dy * dy + dz * dz > pre * pre) continue;
      }
      for (int b = 0; b < G2.ns; ++b)
        for (int s = 0; s < ns; ++s) {
          double ex = mc.pos[0][s][0] - q[3 * b], ey = mc.pos[0][s][1] - q[3 * b + 1],
                 ez = mc.pos[0][s][2] - q[3 * b + 2];
          if (S.use_cells) {
            ex -= S.box[0] * round(ex / S.box[0]);
            ey -= S.box[1] * round(ey / S.box[1]);
            ez -= S.box[2] * round(ez / S.box[2]);
          } else {
            const double *r = S.rcell, *c = S.cell;
            double fx = r[0] * ex + r[3] * ey + r[6] * ez, fy = r[1] * ex + r[4] * ey + r[7] * ez,
                   fz = r[2] * ex + r[5] * ey + r[8] * ez;
            fx -= round(fx);
            fy -= round(fy);
            fz -= round(fz);
            ex = c[0] * fx + c[3] * fy + c[6] * fz;
            ey = c[1] * fx + c[4] * fy + c[7] * fz;
            ez = c[2] * fx + c[5] * fy + c[8] * fz;
          }
          if (ex * ex + ey * ey + ez * ez < S.overlap_sq) hit = 1;
        }
    }
  }
  return block_or(hit, B.ev.red_i);
}

// ----------------------------------------------------------------- k-space
// One pass over the k-vectors for npos positions; writes s(k) of position 0
// to snew and of position 1 to sold, accumulates energies and mixing terms.
template <bool F32>
__device__ void kspace(BlockShared<F32> &B, const ChainArrays &CA, int chain,
                       bool exist0, double *E, double (*mix)[kMaxM + 1]) {
  const SysDev &S = B.S;
  const MoveCtx &mc = B.mc;
  const GuestType &G = S.g[mc.g];
  int ns = mc.ns, npos = mc.npos;
  int mol = G.mol;
  bool disp = npos == 2;
  double2 *snew = CA.snew + (size_t)chain * CA.nkmax;
  double2 *sold = CA.sold + (size_t)chain * CA.nkmax;
  const double2 *skg = CA.sk + (size_t)chain * kMaxG * CA.nkmax;
  const float2 *sk32 = CA.sk32 + (size_t)chain * CA.nmt * CA.nkmax;
  double e[2] = {0.0, 0.0};
  double mx[2][kMaxM + 1];
  for (int p = 0; p < 2; ++p)
    for (int m = 0; m <= kMaxM; ++m) mx[p][m] = 0.0;
  float ef[2] = {0.f, 0.f};
  int cnt = 0;
  for (int k = threadIdx.x; k < S.nk; k += kThreads) {
    int4 lmn = __ldg(S.klmn + k);
    int am = abs(lmn.y), an = abs(lmn.z);
    bool cm = lmn.y < 0, cn = lmn.z < 0;
    if constexpr (!F32) {
      double akk = __ldg(S.akk + k);
      // S(k) per molecule type and total
      double2 sfw = __ldg(S.skfw + k);
      double2 stot = sfw;
      double2 sgt[kMaxG];
      for (int g2 = 0; g2 < S.ntpguest; ++g2) {
        sgt[g2] = skg[(size_t)g2 * CA.nkmax + k];
        stot.x += sgt[g2].x;
        stot.y += sgt[g2].y;
      }
      double2 sp[2];
      for (int p = 0; p < npos; ++p) {
        double2 acc = make_double2(0.0, 0.0);
        for (int s = 0; s < ns; ++s) {
          double2 ex = B.ev.pw64[p][s][0][lmn.x];
          double2 ey = B.ev.pw64[p][s][1][am];
          double2 ez = B.ev.pw64[p][s][2][an];
          if (cm) ey.y = -ey.y;
          if (cn) ez.y = -ez.y;
          double2 t = cmul(cmul(ex, ey), ez);
          acc.x += G.q[s] * t.x;
          acc.y += G.q[s] * t.y;
        }
        sp[p] = acc;
      }
      for (int p = 0; p < npos; ++p) {
        double2 su = stot;
        if (disp && p == 0) {  // new position sees S - s_old (gcmc.f:2862-2871)
          su.x -= sp[1].x;
          su.y -= sp[1].y;
        }
        bool exist = disp ? (p == 1) : exist0;
        double sumsqd = sp[p].x * sp[p].x + sp[p].y * sp[p].y;
        double mixterm = 2.0 * sp[p].x * su.x + 2.0 * sp[p].y * su.y;
        if (exist) mixterm = -1.0 * mixterm;
        e[p] += akk * (mixterm + sumsqd);
        double f2 = 2.0 * akk;
        mx[p][S.fw_mol] += f2 * (sp[p].x * sfw.x + sp[p].y * sfw.y);
        for (int g2 = 0; g2 < S.ntpguest; ++g2) {
          int m2 = S.g[g2].mol;
          if (m2 == mol) continue;
          mx[p][m2] += f2 * (sp[p].x * sgt[g2].x + sp[p].y * sgt[g2].y);
        }
      }
      snew[k] = sp[0];
      if (disp) sold[k] = sp[1];
    } else {
      float akk = __ldg(S.akk32 + k);
      float2 stot = sk32[(size_t)S.maxmls * CA.nkmax + k];
      float2 sp[2];
      for (int p = 0; p < npos; ++p) {
        float2 acc = make_float2(0.f, 0.f);
        for (int s = 0; s < ns; ++s) {
          float2 ex = B.ev.pw32[p][s][0][lmn.x];
          float2 ey = B.ev.pw32[p][s][1][am];
          float2 ez = B.ev.pw32[p][s][2][an];
          if (cm) ey.y = -ey.y;
          if (cn) ez.y = -ez.y;
          float2 t = cmul(cmul(ex, ey), ez);
          float q = (float)G.q[s];
          acc.x = fmaf(q, t.x, acc.x);
          acc.y = fmaf(q, t.y, acc.y);
        }
        sp[p] = acc;
      }
      for (int p = 0; p < npos; ++p) {
        float2 su = stot;
        if (disp && p == 0) {
          su.x -= sp[1].x;
          su.y -= sp[1].y;
        }
        bool exist = disp ? (p == 1) : exist0;
        float sumsqd = fmaf(sp[p].x, sp[p].x, sp[p].y * sp[p].y);
        float mixterm = 2.0f * fmaf(sp[p].x, su.x, sp[p].y * su.y);
        if (exist) mixterm = -mixterm;
        ef[p] = fmaf(akk, mixterm + sumsqd, ef[p]);
        float f2 = 2.0f * akk;
        for (int m2 = 1; m2 <= S.maxmls; ++m2) {
          if (m2 == mol) continue;
          float2 si2 = sk32[(size_t)(m2 - 1) * CA.nkmax + k];
          mx[p][m2] += (double)(f2 * fmaf(sp[p].x, si2.x, sp[p].y * si2.y));
        }
      }
      snew[k] = make_double2(sp[0].x, sp[0].y);
      if (disp) sold[k] = make_double2(sp[1].x, sp[1].y);
      if (++cnt == 8) {
        e[0] += ef[0];
        e[1] += ef[1];
        ef[0] = ef[1] = 0.f;
        cnt = 0;
      }
    }
  }
  if constexpr (F32) {
    e[0] += ef[0];
    e[1] += ef[1];
  }
  for (int p = 0; p < 2; ++p) {
    E[p] = e[p];
    for (int m = 0; m <= kMaxM; ++m) mix[p][m] = mx[p][m];
  }
}

// --------------------------------------------------------------- evaluate
// Evaluate the proposed move; fills mc.estep, mc.delE, flags.  Returns 1 if
// a full evaluation ran (no overlap exit).
template <bool F32>
__device__ int evaluate(BlockShared<F32> &B, const ChainArrays &CA, int chain, int &st) {
  SysDev &S = B.S;
  MoveCtx &mc = B.mc;
  const GuestType &G = S.g[mc.g];
  int ns = mc.ns;
  // site data to shared memory
  if (threadIdx.x < ns) {
    int s = threadIdx.x;
    B.si[s].q = G.q[s];
    B.si[s].chgea = G.q[s] / S.epsq * kR4pie0;
    B.si[s].type = G.type[s];
  }
  if (threadIdx.x < 2 * kMaxS) {
    int p = threadIdx.x / kMaxS, s = threadIdx.x % kMaxS;
    if (p < mc.npos && s < ns) {
      for (int d = 0; d < 3; ++d) {
        double v = mc.pos[p][s][d];
        B.ev.p64[p][s][d] = v;
        float h = (float)v;
        B.ev.phi[p][s][d] = h;
        B.ev.plo[p][s][d] = (float)(v - (double)h);
      }
    }
  }
  __syncthreads();
  bool needs_ov = (mc.kind == 1 || mc.kind >= 3);
  if (needs_ov) {
    int hit = overlap_check(B, CA, chain);
    if (hit) {
      if (threadIdx.x == 0) mc.overlap = 1;
      __syncthreads();
      return 0;
    }
  }
  // ---- pair sums, one position at a time
  Acc acc[2];
  for (int p = 0; p < 2; ++p) {
    acc[p].e2_fw = acc[p].vdw_fw = acc[p].recip = 0.0;
    for (int g2 = 0; g2 < kMaxG; ++g2) acc[p].e2_g[g2] = acc[p].vdw_g[g2] = 0.0;
    for (int m = 0; m <= kMaxM; ++m) acc[p].mix[m] = 0.0;
  }
  int sf[2] = {0, 0}, ovd = 0;
  for (int p = 0; p < mc.npos; ++p) {
    double c[3] = {0, 0, 0};
    for (int s = 0; s < ns; ++s)
      for (int d = 0; d < 3; ++d) c[d] += B.ev.p64[p][s][d];
    for (int d = 0; d < 3; ++d) c[d] /= ns;
    double rm = 0.0;
    for (int s = 0; s < ns; ++s) {
      double dx = B.ev.p64[p][s][0] - c[0], dy = B.ev.p64[p][s][1] - c[1],
             dz = B.ev.p64[p][s][2] - c[2];
      rm = fmax(rm, sqrt(dx * dx + dy * dy + dz * dz));
    }
    build_segments<F32>(S, B.ev, c, S.rcut + rm + 1e-6, st);
    scan_framework<F32>(S, B.ev, p, ns, B.si, acc[p], ovd, sf[p], st);
    __syncthreads();
    scan_guests<F32>(S, B.H, CA, chain, B.ev, p, ns, mc.g, mc.slot, rm, B.si, acc[p], ovd,
                     sf[p], st);
    __syncthreads();
  }
  // ---- k-space
  build_powers<F32>(S, B.ev, mc.npos, ns);
  __syncthreads();
  double E[2], mix[2][kMaxM + 1];
  kspace<F32>(B, CA, chain, mc.kind == 2, E, mix);
  // ---- reduce: per position 2 + 2*G + 1 + maxmls values
  const int nper = 2 + 2 * kMaxG + 1 + (kMaxM + 1);
  double vals[2 * nper];
  for (int p = 0; p < 2; ++p) {
    double *v = vals + p * nper;
    v[0] = acc[p].e2_fw;
    v[1] = acc[p].vdw_fw;
    for (int g2 = 0; g2 < kMaxG; ++g2) {
      v[2 + g2] = acc[p].e2_g[g2];
      v[2 + kMaxG + g2] = acc[p].vdw_g[g2];
    }
    v[2 + 2 * kMaxG] = E[p];
    for (int m = 0; m <= kMaxM; ++m) v[3 + 2 * kMaxG + m] = mix[p][m];
  }
  block_sum(vals, 2 * nper, B.ev.red);
  int sfa = block_or(sf[0], B.ev.red_i);
  int sfb = block_or(sf[1], B.ev.red_i);
  if (threadIdx.x == 0) {
    const double *R = B.ev.red + kWarps * 2 * nper;
    mc.surf_new = sfa;  // position 0
    mc.surf_old = sfb;
    int mol = G.mol;
    double chgtmp = 0.0, sq = 0.0;
    for (int s = 0; s < ns; ++s) {
      chgtmp += G.q[s];
      sq += G.q[s] * G.q[s];
    }
    double r4 = kR4pie0 / S.epsq;
    double engsic0 = -r4 * S.alpha * sq / kSqrPi;
    double sumchg = B.H.sumchg;
    // per position: ewld1, ewald1en(mol,i), ewald2, vdw, ewald2en, vdwen
    double ewld1[2], e2[2], vd[2], e1en[2][kMaxM + 1], e2en[2][kMaxM + 1], vden[2][kMaxM + 1];
    for (int p = 0; p < mc.npos; ++p) {
      const double *v = R + p * nper;
      bool exist = (mc.npos == 2) ? (p == 1) : (mc.kind == 2);
      double qfix = -(0.5 * kPi * r4) *
                    ((chgtmp * sumchg) / S.alpha + (chgtmp / S.alpha) * (chgtmp / S.alpha)) / S.volm;
      double sic = engsic0;
      if (exist) {
        sic = -sic;
        qfix = -qfix;
      }
      ewld1[p] = S.krecip * v[2 + 2 * kMaxG] + sic + qfix;
      e2[p] = v[0];
      vd[p] = v[1];
      for (int m = 0; m <= kMaxM; ++m) e1en[p][m] = e2en[p][m] = vden[p][m] = 0.0;
      e2en[p][S.fw_mol] = v[0];
      vden[p][S.fw_mol] = v[1];
      for (int g2 = 0; g2 < S.ntpguest; ++g2) {
        e2[p] += v[2 + g2];
        vd[p] += v[2 + kMaxG + g2];
        e2en[p][S.g[g2].mol] += v[2 + g2];
        vden[p][S.g[g2].mol] += v[2 + kMaxG + g2];
      }
      for (int m = 1; m <= S.maxmls; ++m) {
        if (m == mol) continue;
        double qfm = -(1.0 * kPi * r4) * (B.H.chgsum_mol[m] * chgtmp) / (S.alpha * S.alpha * S.volm);
        if (exist) qfm = -qfm;
        e1en[p][m] = S.krecip * v[3 + 2 * kMaxG + m] + qfm;
      }
    }
    double e3 = G.ewald3en, eu = S.engunit;
    for (int m = 0; m <= kMaxM; ++m) mc.delE[m] = 0.0;
    if (mc.kind == 1) {
      double delrc;
      gst_lrc(S, B.H, mc.g, false, delrc, mc.delrc_mol);
      mc.delrc = delrc;
      mc.estep = (ewld1[0] + e2[0] - e3 + vd[0] + delrc) / eu;
      for (int m = 1; m <= S.maxmls; ++m)
        if (m != mol) mc.delE[m] = (e1en[0][m] + e2en[0][m] + vden[0][m] + mc.delrc_mol[m]) / eu;
      mc.delE[mol] = mc.estep;
    } else if (mc.kind == 2) {
      double delrc;
      gst_lrc(S, B.H, mc.g, true, delrc, mc.delrc_mol);
      mc.delrc = delrc;
      double est = (-ewld1[0] + e2[0] + vd[0] - e3) / eu;
      mc.estep = est - delrc / eu;
      for (int m = 1; m <= S.maxmls; ++m)
        if (m != mol) mc.delE[m] = -(e1en[0][m] + e2en[0][m] + vden[0][m] + mc.delrc_mol[m]) / eu;
      mc.delE[mol] = -mc.estep;
    } else {
      double enginit = (-ewld1[1] + e2[1] + vd[1] - e3) / eu;
      double enew = (ewld1[0] + e2[0] + vd[0] - e3) / eu;
      mc.estep = enew - enginit;
      mc.delrc = 0.0;
      for (int m = 1; m <= S.maxmls; ++m)
        if (m != mol)
          mc.delE[m] = (e1en[0][m] - e1en[1][m] + e2en[0][m] - e2en[1][m] + vden[0][m] - vden[1][m]) / eu;
      mc.delE[mol] = mc.estep;
    }
    mc.parts[0] = ewld1[0];
    mc.parts[1] = e2[0];
    mc.parts[2] = vd[0];
    mc.parts[3] = mc.delrc;
    mc.ewld1_b = mc.npos == 2 ? ewld1[1] : 0.0;
    mc.chgtmp = chgtmp;
    mc.engsictmp = engsic0;
    if (!isfinite(mc.estep)) st |= kStNonFinite;
  }
  __syncthreads();
  return 1;
}

// ----------------------------------------------------------------- decide
// Thread 0.  rande < 0 asks for a draw from the chain's generator.
template <bool F32>
__device__ void decide(BlockShared<F32> &B, bool draw) {
  MoveCtx &mc = B.mc;
  ChainHdr &H = B.H;
  if (mc.kind == 0) {
    mc.accepted = 0;
    return;
  }
  if (mc.kind == 1) {
    if (mc.overlap) {
      mc.accepted = 0;
      return;
    }
    if (draw) mc.rande = duni_next(H);
    mc.accepted = energy_eval(B.S, H, mc.g, mc.estep, mc.rande, 1);
  } else if (mc.kind == 2) {
    if (draw) mc.rande = duni_next(H);
    mc.accepted = energy_eval(B.S, H, mc.g, -mc.estep, mc.rande, 2);
  } else {
    if (mc.overlap) {
      mc.accepted = 0;
      return;
    }
    if (mc.estep < 0.0) {
      mc.accepted = 1;
      if (draw) mc.rande = -1.0;
    } else {
      if (draw) mc.rande = duni_next(H);
      mc.accepted = energy_eval(B.S, H, mc.g, mc.estep, mc.rande, mc.kind);
    }
  }
}

// Refresh the FP32 mirror of S(k) for k (guest type g changed).
template <bool F32>
__device__ __forceinline__ void refresh_mirror(const SysDev &S, const ChainArrays &CA, int chain,
                                               int k) {
  const double2 *skg = CA.sk + (size_t)chain * kMaxG * CA.nkmax;
  float2 *sk32 = CA.sk32 + (size_t)chain * CA.nmt * CA.nkmax;
  double2 fw = __ldg(S.skfw + k);
  double tx = fw.x, ty = fw.y;
  sk32[(size_t)(S.fw_mol - 1) * CA.nkmax + k] = make_float2((float)fw.x, (float)fw.y);
  for (int g2 = 0; g2 < S.ntpguest; ++g2) {
    double2 v = skg[(size_t)g2 * CA.nkmax + k];
    tx += v.x;
    ty += v.y;
    sk32[(size_t)(S.g[g2].mol - 1) * CA.nkmax + k] = make_float2((float)v.x, (float)v.y);
  }
  sk32[(size_t)S.maxmls * CA.nkmax + k] = make_float2((float)tx, (float)ty);
}

// ----------------------------------------------------------------- commit
// accept_move (mc_moves.f:485-621) for the evaluated move, if accepted.
template <bool F32>
__device__ void commit(BlockShared<F32> &B, const ChainArrays &CA, int chain, int &st) {
  SysDev &S = B.S;
  ChainHdr &H = B.H;
  MoveCtx &mc = B.mc;
  const int accepted = mc.accepted;
  __syncthreads();  // every thread has read the decision before anyone moves on
  if (!accepted) return;
  const GuestType &G = S.g[mc.g];
  int g = mc.g;
  double2 *skg = CA.sk + ((size_t)chain * kMaxG + g) * CA.nkmax;
  const double2 *snew = CA.snew + (size_t)chain * CA.nkmax;
  const double2 *sold = CA.sold + (size_t)chain * CA.nkmax;
  for (int k = threadIdx.x; k < S.nk; k += kThreads) {
    double2 v = skg[k];
    double2 n = snew[k];
    if (mc.kind == 1) {
      v.x += n.x;
      v.y += n.y;
    } else if (mc.kind == 2) {
      v.x -= n.x;
      v.y -= n.y;
    } else {
      double2 o = sold[k];
      v.x = (v.x - o.x) + n.x;
      v.y = (v.y - o.y) + n.y;
    }
    skg[k] = v;
    if constexpr (F32) refresh_mirror<F32>(S, CA, chain, k);
  }
  // molecule order and coordinates
  int *ord = CA.ord + ((size_t)chain * kMaxG + g) * CA.cap;
  int *freel = CA.freel + ((size_t)chain * kMaxG + g) * CA.cap;
  __shared__ int s_slot;
  if (threadIdx.x == 0) {
    int slot = mc.slot;
    if (mc.kind == 1) {
      if (H.nfree[g] > 0) slot = freel[--H.nfree[g]];
      else if (H.nslots[g] < CA.cap) slot = H.nslots[g]++;
      else {
        st |= kStCapacity;
        slot = -1;
      }
      if (slot >= 0) ord[H.nummols[g]] = slot;
    }
    s_slot = slot;
  }
  __syncthreads();
  int slot = s_slot;
  if (mc.kind == 2) {
    // remove entry choice-1 from the order list (mc_moves.f:574-590)
    int n = H.nummols[g];
    int c0 = mc.choice - 1;
    int vals[16];  // capacity <= 4096 = 16 * kThreads
    int cntv = 0;
    for (int i = c0 + threadIdx.x; i < n - 1; i += kThreads) vals[cntv++] = ord[i + 1];
    __syncthreads();
    cntv = 0;
    for (int i = c0 + threadIdx.x; i < n - 1; i += kThreads) ord[i] = vals[cntv++];
    __syncthreads();
  }
  if (slot >= 0 && (mc.kind == 1 || mc.kind >= 3) && threadIdx.x < G.ns) {
    int s = threadIdx.x;
    size_t b = gslot_base(CA, chain, g, slot) + s;
    for (int d = 0; d < 3; ++d) CA.gpos[b * 3 + d] = mc.pos[0][s][d];
    float hx = (float)mc.pos[0][s][0], hy = (float)mc.pos[0][s][1], hz = (float)mc.pos[0][s][2];
    CA.ghi[b] = make_float4(hx, hy, hz, (float)G.q[s]);
    CA.glo[b] = make_float4((float)(mc.pos[0][s][0] - hx), (float)(mc.pos[0][s][1] - hy),
                            (float)(mc.pos[0][s][2] - hz), 0.f);
  }
  if (threadIdx.x == 0 && slot >= 0) {
    for (int m = 1; m <= S.maxmls; ++m) H.energy[m] += mc.delE[m];
    int mol = G.mol;
    if (mc.kind == 1) {
      H.chgsum_mol[mol] += mc.chgtmp;
      H.sumchg += mc.chgtmp;
      if (mc.surf_new) H.surfacemols[mol] += 1;
      for (int s = 0; s < G.ns; ++s) {
        int ka = G.type[s];
        H.numtyp[ka]++;
        H.numtyp_mol[mol][ka]++;
        if (G.frz[s]) {
          H.numfrz[ka]++;
          H.numfrz_mol[mol][ka]++;
        }
      }
      H.nummols[g]++;
    } else if (mc.kind == 2) {
      H.chgsum_mol[mol] -= mc.chgtmp;
      H.sumchg -= mc.chgtmp;
      if (mc.surf_new) H.surfacemols[mol] -= 1;
      for (int s = 0; s < G.ns; ++s) {
        int ka = G.type[s];
        H.numtyp[ka]--;
        H.numtyp_mol[mol][ka]--;
        if (G.frz[s]) {
          H.numfrz[ka]--;
          H.numfrz_mol[mol][ka]--;
        }
      }
      H.nummols[g]--;
      freel[H.nfree[g]++] = slot;
    } else {
      // surface molecule tally of a displacement (gcmc.f:1900-1906)
      if (mc.surf_old && !mc.surf_new) {
        H.surfacemols[mol] -= 1;
        if (H.surfacemols[mol] < 0) H.surfacemols[mol] = 0;
      } else if (!mc.surf_old && mc.surf_new) {
        H.surfacemols[mol] += 1;
      }
    }
  }
  __syncthreads();
}

__device__ inline double calc_qst(double E, double N, double N2, double EN, double T) {
  double d = N2 - N * N;
  return fabs(d) > 0.0 ? -1.0 * (EN - E * N) / d + kRgas * T : 0.0;
}
__device__ inline double calc_cv(double E2, double E, double N, double N2, double EN, double T) {
  double d = N2 - N * N;
  if (fabs(d) > 0.0 && N > 0.0)
    return (3.0 / 2.0 * kRgas) + (E2 - E * E - (EN - E * N) * (EN - E * N) / d) /
                                     (N * 1.9872041e-3 * T * T);
  return 0.0;
}

// Thread 0: acceptance counters and production statistics.
template <bool F32>
__device__ void stats(BlockShared<F32> &B) {
  SysDev &S = B.S;
  ChainHdr &H = B.H;
  MoveCtx &mc = B.mc;
  int g = mc.g;
  if (mc.accepted) {
    if (mc.kind == 1) H.accept_ins[g]++;
    else if (mc.kind == 2) H.accept_del[g]++;
    else if (mc.kind == 4) H.accept_tran[g]++;
    else if (mc.kind == 5) H.accept_rota[g]++;
    else H.accept_disp[g]++;
  }
  if (mc.kind >= 1) {
    H.attempts[mc.kind - 1]++;
    if (mc.accepted) H.accepts[mc.kind - 1]++;
  }
  H.moves++;
  if (!H.production) return;
  if (S.laccsample && !mc.accepted) return;
  H.prodcount++;
  H.rollcount++;
  for (int i = 0; i < S.ntpguest; ++i) {
    int m = S.g[i].mol;
    double dm = double((float)H.nummols[i]);
    double e = H.energy[m];
    double sm = double((float)H.surfacemols[m]);
    H.chainstats[i][0] += dm;
    H.chainstats[i][1] += e;
    H.chainstats[i][2] += e * dm;
    H.chainstats[i][3] += dm * dm;
    H.chainstats[i][4] += e * e;
    H.chainstats[i][5] += sm;
  }
  if (H.prodcount % S.nwindsteps == 0) {
    double rc = double(H.rollcount);
    H.wsum += rc;
    for (int i = 0; i < S.ntpguest; ++i) {
      double aN = H.chainstats[i][0] / rc, E = H.chainstats[i][1] / rc,
             EN = H.chainstats[i][2] / rc, N2 = H.chainstats[i][3] / rc,
             E2 = H.chainstats[i][4] / rc, NF = H.chainstats[i][5] / rc;
      double w[8] = {aN, E, EN, N2, E2, NF, calc_qst(E, aN, N2, EN, S.temp),
                     calc_cv(E2, E, aN, N2, EN, S.temp)};
      for (int q = 0; q < 8; ++q) H.wacc[i][q] += rc * w[q];
      for (int q = 0; q < 6; ++q) H.chainstats[i][q] = 0.0;
    }
    H.windows++;
    H.rollcount = 0;
  }
}

}  // namespace fmcdev

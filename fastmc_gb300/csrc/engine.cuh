// engine.cuh -- the GCMC move loop of one chain on one CTA.
//
// Phases of one main-loop iteration (gcmc.f:704-1164):
//   propose  (warp 0)   lane 0 draws from the MZT generator and picks the
//                       guest and the move (gcmc.f:806-900); the lanes of
//                       warp 0 then build the trial geometry together
//                       (random_ins / random_disp / random_rot / translate /
//                       rotation, utility_pack.f:3161-3563);
//   evaluate (all)      overlap pre-check, pair scans, k-space, fixed-order
//                       reductions, estep and delE as the reference forms
//                       them (mc_moves.f:150-484, gcmc.f:2816-2901);
//   decide   (thread 0) energy_eval (utility_pack.f:3637-3693);
//   commit   (all)      accept_move (mc_moves.f:485-621): S(k), molecule
//                       order, coordinates, counters;
//   stats    (thread 0) production averages and windows (gcmc.f:1050-1128).
//
// GB300 executes FP64 at a small fraction of its FP32 rate, so every phase
// keeps FP64 instructions off the per-pair and per-k loops: positions are
// FP64 (parity of the geometry), pair and k-space terms are FP32 on the FP32
// path, and that path's sums and running S(k) are error-free FP32 hi/lo
// pairs (about 48 significant bits).
#pragma once

#include "device_eval.cuh"

namespace fmcdev {

// Per-phase device clocks of the move loop (built with FMC_PHASE_TIMERS,
// e.g. FMC_PHASE_TIMERS=1 python -m fastmc_gb300.build --force): thread 0
// of each CTA adds the cycles since the previous mark to phase n of its
// chain record; the stats report rank 0's sums.  Compiled out otherwise.
// Phases: 0 proposal, 1 overlap test, 2 neighbour segments and near-guest
// list, 3 framework and guest pair terms, 4 power tables, 5 k-space,
// 6 block reduction, 7 cluster exchange, 8 epilogue, 9 decision and log,
// 10 commit, 11 statistics; speculative rounds: 12 draws and selections,
// 13 first-pass positions, 14 batched overlap tests, 15 exits and the
// round's move.
#ifdef FMC_PHASE_TIMERS
#define FMC_PHASE(B, n)                                     \
  do {                                                      \
    if (threadIdx.x == 0) {                                 \
      const long long t_ = clock64();                       \
      (B).H.phase_cycles[n] += t_ - (B).tmark;              \
      (B).tmark = t_;                                       \
    }                                                       \
  } while (0)
#define FMC_PHASE_SYNC(B, n) \
  do {                       \
    __syncthreads();         \
    FMC_PHASE(B, n);         \
  } while (0)
#else
#define FMC_PHASE(B, n) \
  do {                  \
  } while (0)
#define FMC_PHASE_SYNC(B, n) \
  do {                       \
  } while (0)
#endif

struct LogRec {  // mirrors fmc_move_log
  int move, iguest, choice, overlap, accepted, nmols_after;
  double estep, rande;
  double newxyz[9];
};

constexpr int kMaxSpec = 8;  // proposals of one speculative round
// Widom trials each warp screens between the block's barriers (8 measured
// no faster than 1 on the 102.4 A benchmark: the clear trials' full
// evaluations set the pace)
constexpr int kScreenPer = 1;

// Parallelepiped cells (imcon 3) are compiled into the FP64 kernel and the
// multi-type FP32 kernel; the single-type FP32 kernel (orthorhombic batches)
// carries no code for them, which keeps its registers for the hot loop.
template <bool F32, int GN>
constexpr bool kTricOk = !F32 || GN > 1;

template <bool F32>
struct BlockShared {
  // FP32 batches of one guest type: every guest site in molecule order as
  // hi/lo pairs (x, y, z, q), for the whole launch (ChainArrays::resident)
  float4 grh[F32 ? kGuestSmem : 1];
  float4 grl[F32 ? kGuestSmem : 1];
  SysDev S;
  ChainHdr H;
  MoveCtx mc;
  EvalSmem<F32> ev;
  SiteInfo si[kMaxS];
  int si_g;          // guest type si[] holds (-1: none yet)
  // FP64 bookkeeping of the previous move (energies, charges, production
  // sums), done by thread 32 while warp 0 proposes the next move
  struct Deferred {
    int pending, kind, g, npos, accepted, booked, other, surf_new, surf_old, production, n_old;
    double chgtmp;
    double delE[kMaxM + 1];
  } dfr;
  // a swap or switch move in flight (swap_move, switch_move): the partner
  // type, the new molecule's sites, the energy changes, and the state a
  // rejection puts back; a switch also keeps the partner molecule, both
  // molecules' centres, their sites relative to them and their coordinates
  // before the move (index 0 the chosen molecule, 1 the partner)
  struct Swap {
    int gj, overlap, accepted;
    double estepi, estepj, rande;
    double pos[kMaxS][3];
    int nummols[kMaxG], nslots[kMaxG], nfree[kMaxG], skb[kMaxG];
    double energy[kMaxM + 1], chgsum_mol[kMaxM + 1], surfacemols[kMaxM + 1];
    int numtyp[kMaxT + 1], numfrz[kMaxT + 1];
    int numtyp_mol[kMaxM + 1][kMaxT + 1], numfrz_mol[kMaxM + 1][kMaxT + 1];
    int jchoice, slot_j;
    double cen[2][3], rel[2][kMaxS][3], opos[2][kMaxS][3];
    float4 ohi[2][kMaxS], olo[2][kMaxS];
  } swp;
  // speculative proposals (spec_round): each one's selection, first-pass
  // positions and overlap outcome, and the selection state after it
  struct SelState {
    long long gcmccount, ins, del, disp, tran, rota, jump;
    int minchk_left, production, disp_mod, tran_mod, rota_mod, rhead, ravail, status;
    double delrdisp, tran_delr, rotangle, rota_rotangle;
    float sh_disp[2], sh_tran[2], rho_rot[2][2];
  };
  struct Spec {
    int kind, choice, slot, npos, flag2, flag5, production, testable, hit;
    float draws[7], stepf[4];
    float phi[2][kMaxS][3], plo[2][kMaxS][3];
    SelState sel;
  } spec[kMaxSpec];
  int spec_n, spec_exits, spec_have;
  // Widom jobs: each warp's trial, screened against the framework
  struct WidomScreen {
    float pos[kWarps][kMaxS][3];  // the trial's sites in FP32
    float cell[9], tmpl[kMaxS][3];  // the cell vectors and the guest's sites in float
    int list[kScreenPer][kWarps];  // per round and warp: the trial the screen left, else -1
    int nscreened;
  } wsc;
  float draws[8];
  float stepf[4];    // FP32 path: shift half-width and half-angle / pi scale, hi/lo
  float4 trig[kTrigN];  // FP32 path: the quaternion table (copied per launch)
  double geo[12];    // a, b, c, q1..q4, rotation angle, com/frac scratch
  double vtmp[3];
  int flags[8];     // 0 status, 1 slot, 2 "translate" (q = 0), 3 FP32 geometry, 4 delE deferred,
                    // 5 switch no-op, 6 overlap test already passed (speculative round),
                    // 7 positions out of range (position_bounds)
  // cluster exchange (chains on more than one CTA): per-CTA partial totals,
  // double-buffered, and the flags the peers raise in this CTA's memory
  double xv[2][40];
  unsigned xflag[kMaxCluster];  // xflag[q]: last exchange CTA q has posted here
  unsigned cflag;               // last commit rank 0 has finished
  unsigned xseq, cseq;          // exchanges and commits done (same in every CTA)
  long long tmark;              // FMC_PHASE: clock of the previous mark
};

// Sum ev.out[0..nv) over the CTAs of the chain's cluster, in rank order (so
// every CTA gets the same bits).  All threads; no-op on a single CTA.
template <bool F32>
__device__ void cluster_exchange(BlockShared<F32> &B, int nv, int &st) {
  const int C = B.ev.csize, r = B.ev.rank;
  if (C == 1) return;
  const unsigned n = B.xseq + 1;
  const int par = n & 1;
  for (int i = threadIdx.x; i < nv; i += kThreads) B.xv[par][i] = B.ev.out[i];
  __syncthreads();
  if (threadIdx.x == 0) {
    B.xseq = n;
    for (int q = 0; q < C; ++q)
      if (q != r) dsmem_store_release(dsmem_addr(&B.xflag[r], q), n);
    for (int q = 0; q < C; ++q)
      if (q != r && !wait_flag(&B.xflag[q], n)) st |= kStWait;
  }
  __syncthreads();
  if (threadIdx.x < nv) {
    const int i = threadIdx.x;
    double v[kMaxCluster];
#pragma unroll
    for (int q = 0; q < kMaxCluster; ++q)  // all loads in flight, then the sum in rank order
      v[q] = q >= C ? 0.0 : (q == r ? B.xv[par][i] : dsmem_load_f64(dsmem_addr(&B.xv[par][i], q)));
    double sum = 0.0;
#pragma unroll
    for (int q = 0; q < kMaxCluster; ++q)
      if (q < C) sum += v[q];
    B.ev.out[i] = sum;
  }
  __syncthreads();
}

// After an accepted commit: rank 0 has written the chain's guest arrays;
// the other CTAs wait until those writes are visible before they read them.
template <bool F32>
__device__ void cluster_commit_sync(BlockShared<F32> &B, int &st) {
  const int C = B.ev.csize;
  if (C == 1) return;
  if (B.ev.rank == 0) __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned n = ++B.cseq;
    if (B.ev.rank == 0) {
      for (int q = 1; q < C; ++q) dsmem_store_release(dsmem_addr(&B.cflag, q), n);
    } else if (!wait_flag(&B.cflag, n)) {
      st |= kStWait;
    }
  }
  __syncthreads();
}

__device__ __forceinline__ size_t gslot_base(const ChainArrays &CA, int chain, int g, int slot) {
  return (((size_t)chain * kMaxG + g) * CA.cap + slot) * kMaxS;
}

// gstlrcorrect (vdw_terms.f:686-776) from the host-built coefficients.
__device__ __forceinline__ double lrc_delta(const SysDev &S, const ChainHdr &H, int g,
                                            bool lexisting) {
  const GuestType &G = S.g[g];
  double s = 0.0;
  for (int g2 = 0; g2 < S.ntpguest; ++g2) s += double(H.nummols[g2]) * G.lrcB[g2];
  return lexisting ? (-G.lrcA + 2.0 * G.lrcC - s) : (G.lrcA + s);
}

// energy_eval (utility_pack.f:3637-3693)
template <bool F32>
__device__ inline bool energy_eval(const SysDev &S, const ChainHdr &H, int g, double eng,
                            double rande, int kind) {
  if constexpr (F32) {
    // the same test in log space with FP32 instructions: rande < test
    // <=> log(rande) < log(test); log(prefactor) = lnpf[g] -/+ log(N (+1))
    // with lnpf = log(statvolm * fugacity / (kB T)) set per launch.  At the
    // threshold the FP32 path's own estep error (~1e-7) dominates anyway.
    const float be = (float)S.beta * (float)eng;
    float lnt;
    if (-be > 700.0f) lnt = 700.0f;
    else if (be > 700.0f) lnt = -700.0f;
    else if (kind >= 3) lnt = -be;
    else if (kind == 1) lnt = H.lnpf[g] - logf((float)H.nummols[g] + 1.0f) - be;
    else if (fabs(H.fuga[g]) < 1.0e-7) lnt = 0.0f;
    else lnt = logf((float)H.nummols[g]) - H.lnpf[g] - be;
    return logf((float)rande) < lnt;
  }
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
// Proposal modes.
constexpr int kPropMC = 0;        // main loop: draw guest, move and geometry
constexpr int kPropInsert = 1;    // create molecules: forced insertion of guest g
constexpr int kPropExternal = 2;  // per-move ABI: move given by the host

// Error-free update of one double-float component: (hi, lo) += x.
__device__ __forceinline__ void df_inc(float &hi, float &lo, float x) {
  float s, e;
  two_sum_f(hi, x, s, e);
  e += lo;
  hi = s + e;
  lo = e - (hi - s);
}

// The adaptive step-size updates of gcmc.f:859-900 for guest type g, when
// a count sits at a multiple of 100 (50 for the rotation angle).
template <bool F32>
__device__ __noinline__ void adapt_steps(ChainHdr &H, const GuestType &G, int g) {
  if (H.disp_count[g] >= 1) {
    if (H.disp_mod[g] == 0) {  // disp_count % 100 == 0
      double ratio = double(H.accept_disp[g]) / double(H.disp_count[g]);
      if (ratio > G.disp_ratio) H.delrdisp[g] *= 1.05;
      else if (H.delrdisp[g] > kDelrMin) H.delrdisp[g] *= 0.95;
    } else if (H.disp_mod[g] == 50) {  // disp_count % 50 == 0
      double ratio = double(H.accept_disp[g]) / double(H.disp_count[g]);
      if (ratio > G.disp_ratio) H.rotangle *= 1.05;
      else if (H.rotangle > kMinAngle) H.rotangle *= 0.95;
    }
  }
  if (H.tran_count[g] >= 1 && H.tran_mod[g] == 0) {
    double ratio = double(H.accept_tran[g]) / double(H.tran_count[g]);
    if (ratio > G.tran_ratio) H.tran_delr[g] *= 1.05;
    else if (H.tran_delr[g] > kDelrMin) H.tran_delr[g] *= 0.95;
  }
  if (H.rota_count[g] >= 1 && H.rota_mod[g] == 0) {
    double ratio = double(H.accept_rota[g]) / double(H.rota_count[g]);
    if (ratio > G.rota_ratio) H.rota_rotangle *= 1.05;
    else if (H.rota_rotangle > kMinAngle) H.rota_rotangle *= 0.95;
  }
  if (F32) sync_step_pairs(H, g);
}

// Lane 0 of warp 0: move selection and draws (gcmc.f:806-900, 1693-1870).
template <bool F32>
__device__ void select_move(BlockShared<F32> &B, const ChainArrays &CA, int chain) {
  SysDev &S = B.S;
  ChainHdr &H = B.H;
  MoveCtx &mc = B.mc;
  H.gcmccount++;
  if (--H.minchk_left == 0) {  // gcmccount is a multiple of minchk
    H.minchk_left = S.minchk;
    if (!H.production && S.eqsteps > 0 && H.gcmccount >= S.eqsteps) H.production = 1;
  }
  DrawCursor dc(H);  // this move's draws, buffer position in registers
  int g = 0;
  if (S.ntpguest > 1) g = pick1(dc.next(), S.ntpguest) - 1;
  const GuestType &G = S.g[g];
  int nmols = H.nummols[g];
  float randmov = dc.next();
  int kind;
  if (randmov < G.mcinsf) kind = 1;
  else if (randmov < G.mcdelf) kind = 2;
  else if (randmov < G.mcdisf) kind = 3;
  else if (randmov < G.mcjmpf) kind = 6;  // jump
  else if (randmov < G.mcswpf) kind = 7;  // swap
  else if (randmov < G.mctraf) kind = 4;
  else if (randmov < G.mcrotf) kind = 5;
  else if (randmov < G.mcswif) kind = 8;  // switch
  else kind = 3;
  // adaptive step sizes (gcmc.f:859-900); the updates themselves (FP64) are
  // out of line, the tests here are integer compares
  if (nmols >= 1 && ((H.disp_count[g] >= 1 && (H.disp_mod[g] == 0 || H.disp_mod[g] == 50)) ||
                     (H.tran_count[g] >= 1 && H.tran_mod[g] == 0) ||
                     (H.rota_count[g] >= 1 && H.rota_mod[g] == 0)))
    adapt_steps<F32>(H, G, g);
  if (nmols == 0) kind = 1;
  int nsw = 0, swg[kMaxG];  // switch_chosen_guest: the other types holding molecules
  if (kind == 8) {
    // mc_switch (gcmc.f:2041-2267) returns before any draw unless two other
    // guest types hold molecules: then no move, and `accepted` keeps its value
    for (int i = 0; i < S.ntpguest; ++i)
      if (H.nummols[i] > 0 && i != g) swg[nsw++] = i;
    if (nsw < 2) {
      B.flags[5] = 1;
      kind = 0;
    }
  }
  mc.kind = kind;
  mc.g = g;
  mc.ns = G.ns;
  mc.choice = 0;
  mc.slot = -1;
  mc.npos = 1;
  if (kind == 1) {
    H.ins_count[g]++;
    for (int i = 0; i < 7; ++i) B.draws[i] = dc.next();  // random_ins
  } else if (kind == 2) {
    H.del_count[g]++;
    mc.choice = pick1(dc.next(), nmols);
  } else if (kind == 7) {
    // mc_swap (gcmc.f:2269-2452): the molecule (floor(duni n + 1)), the
    // partner guest type among the others, then random_rot with the
    // displacement angle (utility_pack.f:3526-3563); run by swap_move
    mc.choice = pick1(dc.next(), nmols);
    const int jg = pick1(dc.next(), S.ntpguest - 1);  // 1-based among the others
    B.swp.gj = jg < g + 1 ? jg - 1 : jg;
    for (int i = 3; i < 7; ++i) B.draws[i] = dc.next();
    B.geo[7] = H.rotangle;
  } else if (kind == 8) {
    // the acting mc_switch (gcmc.f:2096-2107): the partner type among the
    // others holding molecules, then a molecule of each; run by switch_move
    B.swp.gj = swg[pick1(dc.next(), nsw) - 1];
    mc.choice = pick1(dc.next(), nmols);
    B.swp.jchoice = pick1(dc.next(), H.nummols[B.swp.gj]);
  } else if (kind == 6) {
    // mc_jump (gcmc.f:1937-2039): the molecule, then random_jump's point
    // (utility_pack.f:3359-3380) and random_rot with angle 2 pi
    H.jump_count[g]++;
    mc.choice = pick1(dc.next(), nmols);
    for (int i = 0; i < 7; ++i) B.draws[i] = dc.next();
    if constexpr (!F32) B.geo[7] = 2.0 * kPi;
    B.flags[2] = 0;
    mc.npos = 2;
  } else if (kind != 0) {
    double a = 0.0, b = 0.0, c = 0.0;
    B.draws[3] = -1.0f;  // no rotation unless drawn
    if (kind != 5) {     // random_disp (utility_pack.f:3333-3357)
      if constexpr (F32) {  // the draws; the shift is built by the geometry
        for (int i = 0; i < 3; ++i) B.draws[i] = dc.next();
        const float *hp = kind == 4 ? H.sh_tran[g] : H.sh_disp[g];
        B.stepf[0] = hp[0];
        B.stepf[1] = hp[1];
      } else {
        double dd = kind == 4 ? H.tran_delr[g] : H.delrdisp[g];
        double h = dd * 0.5;
        a = (2.0 * (double)dc.next() - 1.0) * h;
        b = (2.0 * (double)dc.next() - 1.0) * h;
        c = (2.0 * (double)dc.next() - 1.0) * h;
      }
    }
    if (kind != 4) {  // random_rot (utility_pack.f:3526-3563)
      for (int i = 3; i < 7; ++i) B.draws[i] = dc.next();
      if constexpr (F32) {
        const float *rp = H.rho_rot[kind == 5 ? 1 : 0];
        B.stepf[2] = rp[0];
        B.stepf[3] = rp[1];
      } else {
        B.geo[7] = kind == 5 ? H.rota_rotangle : H.rotangle;
      }
      B.flags[2] = 0;
    } else {
      // "move translate" keeps q1..q4 = 0 (gcmc.f:1842), and rotation()
      // with a zero quaternion applies Q = -I: the molecule is inverted
      // through its centre of mass.  Reproduced as the reference does it.
      B.geo[3] = B.geo[4] = B.geo[5] = B.geo[6] = 0.0;
      B.draws[3] = 1.0f;
      B.flags[2] = 1;
    }
    if (kind == 4) {
      H.tran_count[g]++;
      if (++H.tran_mod[g] == 100) H.tran_mod[g] = 0;
    } else if (kind == 5) {
      H.rota_count[g]++;
      if (++H.rota_mod[g] == 100) H.rota_mod[g] = 0;
    } else {
      H.disp_count[g]++;
      if (++H.disp_mod[g] == 100) H.disp_mod[g] = 0;
    }
    B.geo[0] = a;
    B.geo[1] = b;
    B.geo[2] = c;
    mc.choice = pick1(dc.next(), nmols);
    mc.npos = 2;
  }
  dc.done();
}

// Quaternion of random_ins / random_rot from four draws and an angle:
// theta = r1 * angle, axis (2 r2 - 1, 2 r3 - 1, 2 r4 - 1) normalised.
__device__ __forceinline__ void draw_quaternion(const float *d, double angle, double *q) {
  double half = 0.5 * ((double)d[3] * angle);
  double sn, cs;
  sincos(half, &sn, &cs);
  double b1 = 2.0 * (double)d[4] - 1.0, b2 = 2.0 * (double)d[5] - 1.0,
         b3 = 2.0 * (double)d[6] - 1.0;
  double rn = 1.0 / sqrt(b1 * b1 + b2 * b2 + b3 * b3);
  q[0] = cs;
  q[1] = sn * (b1 * rn);
  q[2] = sn * (b2 * rn);
  q[3] = sn * (b3 * rn);
}

// Row d of the rotation matrix of rotation() (utility_pack.f:3497-3506).
template <class T>
__device__ __forceinline__ void qrow(const T *q, int d, T *row) {
  T q1 = q[0], q2 = q[1], q3 = q[2], q4 = q[3];
  if (d == 0) {
    row[0] = T(2) * q2 * q2 + T(2) * q1 * q1 - T(1);
    row[1] = T(2) * q2 * q3 - T(2) * q1 * q4;
    row[2] = T(2) * q2 * q4 + T(2) * q1 * q3;
  } else if (d == 1) {
    row[0] = T(2) * q2 * q3 + T(2) * q1 * q4;
    row[1] = T(2) * q1 * q1 + T(2) * q3 * q3 - T(1);
    row[2] = T(2) * q3 * q4 - T(2) * q1 * q2;
  } else {
    row[0] = T(2) * q2 * q4 - T(2) * q1 * q3;
    row[1] = T(2) * q3 * q4 + T(2) * q1 * q2;
    row[2] = T(2) * q4 * q4 + T(2) * q1 * q1 - T(1);
  }
}

// Warp 0: the trial geometry, one lane per site coordinate.
template <bool F32>
__device__ void geometry_warp(BlockShared<F32> &B, const ChainArrays &CA, int chain, int mode) {
  const SysDev &S = B.S;
  MoveCtx &mc = B.mc;
  const int lane = threadIdx.x & 31;
  if (mc.kind == 0 || mc.kind >= 7) return;  // swap_move / switch_move build their positions
  const GuestType &G = S.g[mc.g];
  const int ns = G.ns;
  const bool mine = lane < 3 * ns;
  const int s = lane / 3, d = lane % 3;
  if (mc.kind == 1) {
    if (mode == kPropExternal) return;  // positions given by the host
    // random_ins: centre from three fractions, orientation from four draws
    double q[4], row[3];
    draw_quaternion(B.draws, 2.0 * kPi, q);
    if (mine) {
      qrow(q, d, row);
      const double *t = G.tmpl[s];
      double v = row[0] * t[0] + row[1] * t[1] + row[2] * t[2];
      double cc = (double)B.draws[0] * S.cell[d] + (double)B.draws[1] * S.cell[3 + d] +
                  (double)B.draws[2] * S.cell[6 + d];
      mc.pos[0][s][d] = v + cc;
    }
    return;
  }
  // delete / displace: the molecule's current sites (get_guest)
  const double *src = CA.gpos + gslot_base(CA, chain, mc.g, mc.slot) * 3;
  double old = mine ? src[3 * s + d] : 0.0;
  if (mc.kind == 2) {
    if (mine) mc.pos[0][s][d] = old;
    return;
  }
  if (mc.kind == 6) {
    // jump: the translation from the old centre of mass to the drawn point
    if (mine) mc.pos[1][s][d] = old;
    __syncwarp();
    if (lane < 3) {
      double cm = 0.0;
      for (int k = 0; k < ns; ++k) cm += mc.pos[1][k][lane] * G.mass[k];
      const double cart = (double)B.draws[0] * S.cell[lane] + (double)B.draws[1] * S.cell[3 + lane] +
                          (double)B.draws[2] * S.cell[6 + lane];
      B.geo[lane] = cart - cm * G.rmass;
    }
    __syncwarp();
  }
  // translate (utility_pack.f:3161-3218): shift, wrap the centre of mass
  if (mine) {
    mc.pos[1][s][d] = old;
    mc.pos[0][s][d] = B.geo[d] + old;
  }
  __syncwarp();
  if (lane < 3) {  // centre of mass
    double cm = 0.0;
    for (int k = 0; k < ns; ++k) cm += mc.pos[0][k][lane] * G.mass[k];
    B.vtmp[lane] = cm * G.rmass;
  }
  __syncwarp();
  if (lane < 3) {
    const double *r = S.rcell;
    double f = r[lane] * B.vtmp[0] + r[3 + lane] * B.vtmp[1] + r[6 + lane] * B.vtmp[2];
    B.geo[8 + lane] = f - floor(f);
  }
  __syncwarp();
  double w = S.cell[d] * B.geo[8] + S.cell[3 + d] * B.geo[9] + S.cell[6 + d] * B.geo[10];
  if (mine) mc.pos[0][s][d] += w - B.vtmp[d];
  __syncwarp();
  // rotation about the wrapped centre (gcmc.f:2876)
  if (B.draws[3] >= 0.0f) {
    double q[4], row[3];
    if (mode == kPropExternal || B.flags[2]) {
      q[0] = B.geo[3];
      q[1] = B.geo[4];
      q[2] = B.geo[5];
      q[3] = B.geo[6];
    } else {
      draw_quaternion(B.draws, B.geo[7], q);
    }
    double wx = S.cell[0] * B.geo[8] + S.cell[3] * B.geo[9] + S.cell[6] * B.geo[10];
    double wy = S.cell[1] * B.geo[8] + S.cell[4] * B.geo[9] + S.cell[7] * B.geo[10];
    double wz = S.cell[2] * B.geo[8] + S.cell[5] * B.geo[9] + S.cell[8] * B.geo[10];
    double x = 0, y = 0, z = 0;
    if (mine) {
      x = mc.pos[0][s][0] - wx;
      y = mc.pos[0][s][1] - wy;
      z = mc.pos[0][s][2] - wz;
    }
    __syncwarp();
    if (mine) {
      qrow(q, d, row);
      double wd = d == 0 ? wx : (d == 1 ? wy : wz);
      mc.pos[0][s][d] = (row[0] * x + row[1] * y + row[2] * z) + wd;
    }
  }
}

// Centre and bounding radius of each evaluated position from its FP32
// coordinates; all lanes of one warp, lane 3p + d takes coordinate d of
// position p (the radius carries a 1e-3 A margin).
template <bool F32>
__device__ __forceinline__ void position_bounds(BlockShared<F32> &B, int lane) {
  const unsigned full = 0xffffffffu;
  const int ns = B.mc.ns, npos = B.mc.npos;
  const int p = lane / 3, d = lane - 3 * (lane / 3);
  const bool act = lane < 3 * npos;
  float c = 0.f;
  if (act) {
    for (int s = 0; s < ns; ++s) c += B.ev.phi[p][s][d];
    c *= B.S.g[B.mc.g].rns;
  }
  float rm2 = 0.f;
  const int b = act ? 3 * p : 0;
  for (int s = 0; s < ns; ++s) {
    const float dd = act ? B.ev.phi[p][s][d] - c : 0.f;
    const float q = dd * dd;
    const float t = __shfl_sync(full, q, b) + __shfl_sync(full, q, b + 1) + __shfl_sync(full, q, b + 2);
    rm2 = fmaxf(rm2, t);
  }
  if (act) B.ev.cen[p][d] = c;
  if (act && d == 0) B.ev.rmx[p] = sqrtf(rm2) + 1e-3f;
  // positions that are not finite or far outside any cell (a damaged
  // state): the evaluation refuses them before any index is formed
  const unsigned bad = __ballot_sync(full, act && !(fabsf(c) < 1.0e6f && rm2 < 1.0e4f));
  if (lane == 0) B.flags[7] = bad ? 1 : 0;
}

// FP32 quaternion of random_ins / random_rot: half angle pi * r * scale
// (scale = angle / 2 pi), axis (2 r - 1) normalised.
__device__ __forceinline__ void quat_f32(const float *dr, float scale, float *q) {
  float sn, cs;
  sincospif(dr[3] * scale, &sn, &cs);
  const float b1 = 2.0f * dr[4] - 1.0f, b2 = 2.0f * dr[5] - 1.0f, b3 = 2.0f * dr[6] - 1.0f;
  const float rn = rsqrtf(b1 * b1 + b2 * b2 + b3 * b3);
  q[0] = cs;
  q[1] = sn * (b1 * rn);
  q[2] = sn * (b2 * rn);
  q[3] = sn * (b3 * rn);
}

// Parallelepiped cell, FP32 path: coordinate d of cell . u (u fractional,
// three values) as a hi/lo pair, exact products summed without loss.
__device__ __forceinline__ void cart_tric(const SysDev &S, const float *u, int d, float &h,
                                          float &l) {
  h = 0.f;
  l = 0.f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float c = S.cellh[d + 3 * k];
    const float p = u[k] * c;
    const float pe = fmaf(u[k], c, -p) + u[k] * S.celll[d + 3 * k];
    float t, e;
    two_sum_f(h, p, t, e);
    h = t;
    l += e + pe;
  }
}

// Coordinate d of cell . n for whole cell translations n (a hi/lo pair).
__device__ __forceinline__ void cell_shift(const SysDev &S, const float *n, int d, float &h,
                                           float &l) {
  cart_tric(S, n, d, h, l);
}

// FP32 path, moves drawn on the device, first pass: geometry_warp's
// construction in plain FP32 arithmetic on hi/lo positions (good to about
// 1e-7 A), for the overlap test that ends most trial moves.  A move that
// passes it gets its positions again from refine_geometry at double-float
// precision before its energy is evaluated.  One warp, one lane per site
// coordinate; orthorhombic cells.  Writes position 0 (new) and, for moves
// of an existing molecule, position 1 (old) into phi/plo; the bounds of
// each position carry a 1e-3 A margin that covers the refinement.
template <bool F32, bool TRIC>
__device__ void geometry_f32_core(const BlockShared<F32> &B, const ChainArrays &CA, int chain,
                                  int kind, int g, int slot, const float *draws, const float *stepf,
                                  int flag2, float (*phi)[kMaxS][3], float (*plo)[kMaxS][3]) {
  const SysDev &S = B.S;
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const GuestType &G = S.g[g];
  const int ns = G.ns;
  const bool mine = lane < 3 * ns;
  const int s = mine ? lane / 3 : 0;
  const int d = lane % 3;
  const float Lh = S.boxh[d], Ll = S.boxl[d];
  float ph = 0.f, pl = 0.f, e;
  if (kind == 1) {
    float q[4], row[3];
    quat_f32(draws, 1.0f, q);
    qrow(q, d, row);
    const float *t = G.tmplf[s];
    const float v = row[0] * t[0] + row[1] * t[1] + row[2] * t[2];
    const float u = draws[d];
    float ch, cl;
    if (!TRIC || S.use_cells) {
      ch = __fmul_rn(u, Lh);
      cl = fmaf(u, Lh, -ch) + u * Ll;
    } else {
      cart_tric(S, draws, d, ch, cl);
    }
    two_sum_f(ch, v, ph, e);
    pl = cl + e;
  } else {
    float oh = 0.f, ol = 0.f;
    if (mine && CA.resident) {
      oh = reinterpret_cast<const float *>(&B.grh[slot * ns + s])[d];
      ol = reinterpret_cast<const float *>(&B.grl[slot * ns + s])[d];
    } else if (mine) {
      const size_t b = gslot_base(CA, chain, g, slot) + s;
      oh = reinterpret_cast<const float *>(CA.ghi + b)[d];
      ol = reinterpret_cast<const float *>(CA.glo + b)[d];
    }
    if (kind == 2) {
      ph = oh;
      pl = ol;
    } else {
      if (mine) {
        phi[1][s][d] = oh;
        plo[1][s][d] = ol;
      }
      // centre of mass of the old molecule, relative to site 0 (jump only)
      const float p0h = __shfl_sync(full, oh, d), p0l = __shfl_sync(full, ol, d);
      float sh = 0.f;
      if (kind == 6) {  // jump: the old centre of mass to the drawn point
        const float off = mine ? ((oh - p0h) + (ol - p0l)) * G.wf[s] : 0.f;
        float cof = 0.f;
        for (int s2 = 0; s2 < ns; ++s2) cof += __shfl_sync(full, off, 3 * s2 + d);
        const float u = draws[d];
        float ch, cl;
        if (!TRIC || S.use_cells) {
          ch = __fmul_rn(u, Lh);
          cl = fmaf(u, Lh, -ch) + u * Ll;
        } else {
          cart_tric(S, draws, d, ch, cl);
        }
        sh = (ch - p0h) + (cl - p0l) - cof;
      } else if (kind != 5) {
        sh = __fmul_rn(2.0f * draws[d] - 1.0f, stepf[0]);
      }
      two_sum_f(oh, sh, ph, e);
      pl = ol + e;
      // centre of mass, relative to site 0, as a hi/lo pair
      const float s0h = __shfl_sync(full, ph, d), s0l = __shfl_sync(full, pl, d);
      const float off = mine ? ((ph - s0h) + (pl - s0l)) * G.wf[s] : 0.f;
      float cof = 0.f;
      for (int s2 = 0; s2 < ns; ++s2) cof += __shfl_sync(full, off, 3 * s2 + d);
      float cmh, cml;
      two_sum_f(s0h, cof, cmh, e);
      cml = s0l + e;
      // wrap the centre into the cell by whole edges (translate)
      if (!TRIC || S.use_cells) {
        const float k = floorf((cmh + cml) * S.rboxf[d]);
        if (k != 0.0f) {
          float t;
          two_sum_f(ph, -k * Lh, t, e);
          ph = t;
          pl += e - k * Ll;
          two_sum_f(cmh, -k * Lh, t, e);
          cmh = t;
          cml += e - k * Ll;
        }
      } else {  // parallelepiped: whole cell translations of the fractional centre
        float c3[3], n[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) c3[j] = __shfl_sync(full, cmh + cml, j);
#pragma unroll
        for (int k = 0; k < 3; ++k)
          n[k] = floorf(fmaf(S.rcellh[k], c3[0], fmaf(S.rcellh[k + 3], c3[1], S.rcellh[k + 6] * c3[2])));
        if (n[0] != 0.f || n[1] != 0.f || n[2] != 0.f) {
          float th, tl, t;
          cell_shift(S, n, d, th, tl);
          two_sum_f(ph, -th, t, e);
          ph = t;
          pl += e - tl;
          two_sum_f(cmh, -th, t, e);
          cmh = t;
          cml += e - tl;
        }
      }
      if (kind == 6 || draws[3] >= 0.0f) {  // rotation about the wrapped centre
        float q[4] = {0.f, 0.f, 0.f, 0.f};  // "move translate": q = 0, Q = -I
        if (kind == 6) quat_f32(draws, 1.0f, q);
        else if (!flag2) quat_f32(draws, stepf[2], q);
        const float x = (ph - cmh) + (pl - cml);
        const float x0 = __shfl_sync(full, x, 3 * s), x1 = __shfl_sync(full, x, 3 * s + 1),
                    x2 = __shfl_sync(full, x, 3 * s + 2);
        float row[3];
        qrow(q, d, row);
        const float v = row[0] * x0 + row[1] * x1 + row[2] * x2;
        two_sum_f(cmh, v, ph, e);
        pl = cml + e;
      }
    }
  }
  if (mine) {
    phi[0][s][d] = ph;
    plo[0][s][d] = pl;
  }
}

// The site constants of the moving guest type and the bounds of the
// evaluated positions (warp 0).
template <bool F32>
__device__ void site_constants_and_bounds(BlockShared<F32> &B) {
  const MoveCtx &mc = B.mc;
  const GuestType &G = B.S.g[mc.g];
  const int lane = threadIdx.x & 31, ns = G.ns;
  if (B.si_g != mc.g) {  // site constants of the moving guest type
    if (lane < ns) {
      SiteInfo &si = B.si[lane];
      si.q = G.q[lane];
      si.chgea = G.chgea[lane];
      si.chgeaf = G.chgeaf[lane];
      si.chgeaf_lo = G.chgeaf_lo[lane];
      si.qf = (float)G.q[lane];
      si.type = G.type[lane];
      si.prow = G.prow[lane];
      si.psig2 = G.psig2[lane];
    }
    __syncwarp();
    if (lane == 0) B.si_g = mc.g;
  }
  __syncwarp();
  position_bounds(B, lane);
}

// FP32 path, moves drawn on the device: the first-pass geometry of the move
// in mc (warp 0), then the site constants and position bounds.
template <bool F32, bool TRIC>
__device__ void geometry_f32(BlockShared<F32> &B, const ChainArrays &CA, int chain) {
  MoveCtx &mc = B.mc;
  if (mc.kind == 0 || mc.kind >= 7) return;  // swap_move / switch_move build their positions
  geometry_f32_core<F32, TRIC>(B, CA, chain, mc.kind, mc.g, mc.slot, B.draws, B.stepf, B.flags[2], B.ev.phi,
                    B.ev.plo);
  __syncwarp();
  site_constants_and_bounds(B);
}

// Double-float quaternion: the half angle pi * rho, rho = r * scale (scale
// = angle / 2 pi), from the table of sin/cos(pi k / 64) at the nearest k
// and the Taylor series of the remainder t (|t| <= pi / 128: sin t = t -
// t^3/6 + t^5/120, cos t = 1 - t^2/2 + t^4/24 - t^6/720, the next terms
// below 2e-15); the axis (2 r - 1, exact in double-float) scaled by 1/|axis|
// from rsqrtf and one Newton step.
__device__ __forceinline__ void quat_df(const float *dr, F2 scale, const float4 *trig, F2 *q) {
  const F2 rho = f2_mulf(scale, dr[3]);
  const float nf = rintf(rho.h * 64.0f);
  float rh, rl;
  two_sum_f(rho.h - nf * 0.015625f, rho.l, rh, rl);  // rho.h - nf/64 is exact
  const float4 T = trig[((int)nf) & (kTrigN - 1)];
  const F2 t = f2_mul(F2{3.14159274f, -8.74227766e-8f}, F2{rh, rl});
  const float t2 = __fmul_rn(t.h, t.h);
  const float s3 = __fmul_rn(t.h, t2) * fmaf(t2, 1.0f / 120.0f, -1.0f / 6.0f);
  const F2 st = f2_addf(t, s3);
  const float tte = fmaf(2.0f * t.h, t.l, fmaf(t.h, t.h, -t2));
  F2 ct = f2_add(F2{1.0f, 0.0f}, F2{-0.5f * t2, -0.5f * tte});
  ct = f2_addf(ct, __fmul_rn(t2, t2) * fmaf(t2, -1.0f / 720.0f, 1.0f / 24.0f));
  const F2 Sk = {T.x, T.y}, Ck = {T.z, T.w};
  const F2 sn = f2_add(f2_mul(Sk, ct), f2_mul(Ck, st));
  const F2 cs = f2_sub(f2_mul(Ck, ct), f2_mul(Sk, st));
  F2 b[3];
  for (int i = 0; i < 3; ++i) two_sum_f(2.0f * dr[4 + i], -1.0f, b[i].h, b[i].l);
  const F2 n2 = f2_add(f2_add(f2_mul(b[0], b[0]), f2_mul(b[1], b[1])), f2_mul(b[2], b[2]));
  const float y = rsqrtf(n2.h);
  const F2 r = f2_mul(n2, f2_mulf(F2{y, 0.0f}, y));
  const float res = (1.0f - r.h) - r.l;
  const F2 rn = f2_addf(F2{y, 0.0f}, __fmul_rn(0.5f * y, res));
  const F2 srn = f2_mul(sn, rn);
  q[0] = cs;
  for (int i = 0; i < 3; ++i) q[i + 1] = f2_mul(srn, b[i]);
}

// Row d of rotation() (utility_pack.f:3497-3506) in double-float.  The ten
// quaternion products are formed on every lane (no divergence on d).
__device__ __forceinline__ void qrow_df(const F2 *q, int d, F2 *row) {
  auto m2 = [](F2 x, F2 y) {
    const F2 p = f2_mul(x, y);
    return F2{2.0f * p.h, 2.0f * p.l};
  };
  const F2 q11 = m2(q[0], q[0]), q22 = m2(q[1], q[1]), q33 = m2(q[2], q[2]), q44 = m2(q[3], q[3]);
  const F2 q12 = m2(q[0], q[1]), q13 = m2(q[0], q[2]), q14 = m2(q[0], q[3]);
  const F2 q23 = m2(q[1], q[2]), q24 = m2(q[1], q[3]), q34 = m2(q[2], q[3]);
  const F2 dg = d == 0 ? q22 : (d == 1 ? q33 : q44);
  const F2 diag = f2_addf(f2_add(dg, q11), -1.0f);
  if (d == 0) {
    row[0] = diag;
    row[1] = f2_sub(q23, q14);
    row[2] = f2_add(q24, q13);
  } else if (d == 1) {
    row[0] = f2_add(q23, q14);
    row[1] = diag;
    row[2] = f2_sub(q34, q12);
  } else {
    row[0] = f2_sub(q24, q13);
    row[1] = f2_add(q34, q12);
    row[2] = diag;
  }
}

// Second pass of the FP32 path's device-drawn geometry, for a move that
// passed the overlap test: geometry_warp's construction in double-float
// (about 48-bit significands), so that the positions agree with the FP64
// construction to ~1e-13 A.  A position error of 1e-7 A (plain FP32)
// would move a repulsive r^-12 term near the overlap distance by ~1e-6
// relative; this one moves it by ~1e-12.  Warp 0, one lane per site
// coordinate; the draws, old positions (phi/plo[1]) and step sizes are the
// first pass's.
template <bool F32, bool TRIC>
__device__ __noinline__ void refine_geometry(BlockShared<F32> &B, const ChainArrays &CA) {
  const SysDev &S = B.S;
  const MoveCtx &mc = B.mc;
  EvalSmem<F32> &ev = B.ev;
  const int lane = threadIdx.x & 31;
  const GuestType &G = S.g[mc.g];
  const int ns = G.ns;
  const bool mine = lane < 3 * ns;
  const int s = mine ? lane / 3 : 0;
  const int d = lane % 3;
  const F2 L = {S.boxh[d], S.boxl[d]};
  const bool free_rot = mc.kind == 1 || mc.kind == 6;  // angle 2 pi
  const bool rot = free_rot || B.draws[3] >= 0.0f;
  F2 q[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};  // "move translate": Q = -I
  if (rot && (free_rot || !B.flags[2]))
    quat_df(B.draws, free_rot ? F2{1.0f, 0.0f} : F2{B.stepf[2], B.stepf[3]}, B.trig, q);
  F2 row[3];
  if (rot) qrow_df(q, d, row);
  auto cart = [&]() {  // the drawn point u * L (cell . u), u = draws[0..2]
    if (TRIC && !S.use_cells) {
      float h, l;
      cart_tric(S, B.draws, d, h, l);
      return f2_norm(h, l);
    }
    const float u = B.draws[d];
    const float ch = __fmul_rn(u, L.h);
    return f2_norm(ch, fmaf(u, L.h, -ch) + __fmul_rn(u, L.l));
  };
  auto com = [&](F2 p) {  // centre of mass, coordinate d (sum of m_k/M x_k)
    F2 c = {0.f, 0.f};
    for (int k = 0; k < ns; ++k) c = f2_add(c, f2_mul(F2{G.wf[k], G.wf_lo[k]}, f2_shfl(p, 3 * k + d)));
    return c;
  };
  auto rotate = [&](F2 x) {  // row d of Q times the site's offset x
    const F2 x0 = f2_shfl(x, 3 * s), x1 = f2_shfl(x, 3 * s + 1), x2 = f2_shfl(x, 3 * s + 2);
    return f2_add(f2_add(f2_mul(row[0], x0), f2_mul(row[1], x1)), f2_mul(row[2], x2));
  };
  F2 p;
  if (mc.kind == 1) {  // random_ins: template rotated about the drawn point
    F2 t = {0.f, 0.f};
    if (mine) t = {G.tmplf[s][d], G.tmplf_lo[s][d]};
    p = f2_add(cart(), rotate(t));
  } else {
    F2 o = {0.f, 0.f};
    if (mine) o = {ev.phi[1][s][d], ev.plo[1][s][d]};
    F2 a = {0.f, 0.f};
    if (mc.kind == 6) {
      a = f2_sub(cart(), com(o));
    } else if (mc.kind != 5) {
      F2 b;
      two_sum_f(2.0f * B.draws[d], -1.0f, b.h, b.l);
      a = f2_mul(b, F2{B.stepf[0], B.stepf[1]});
    }
    p = f2_add(o, a);
    F2 c = com(p);
    if (!TRIC || S.use_cells) {
      const float k = floorf(c.h * S.rboxf[d]);  // wrap the centre into the cell
      if (k != 0.0f) {
        const F2 kL = f2_mulf(L, k);
        p = f2_sub(p, kL);
        c = f2_sub(c, kL);
      }
    } else {  // parallelepiped: whole cell translations of the fractional centre
      const unsigned full = 0xffffffffu;
      float c3[3], n[3];
#pragma unroll
      for (int j = 0; j < 3; ++j) c3[j] = __shfl_sync(full, c.h + c.l, j);
#pragma unroll
      for (int k = 0; k < 3; ++k)
        n[k] = floorf(fmaf(S.rcellh[k], c3[0], fmaf(S.rcellh[k + 3], c3[1], S.rcellh[k + 6] * c3[2])));
      if (n[0] != 0.f || n[1] != 0.f || n[2] != 0.f) {
        float th, tl;
        cell_shift(S, n, d, th, tl);
        const F2 t = f2_norm(th, tl);
        p = f2_sub(p, t);
        c = f2_sub(c, t);
      }
    }
    if (rot) p = f2_add(c, rotate(f2_sub(p, c)));
  }
  if (mine) {
    ev.phi[0][s][d] = p.h;
    ev.plo[0][s][d] = p.l;
  }
}

// Warp 0 proposal for all modes; ends with a block barrier.
template <bool F32, bool TRIC>
__device__ void propose(BlockShared<F32> &B, const ChainArrays &CA, int chain, int mode, int g_forced) {
  if (threadIdx.x < 32) {
    // at least 16 draws in the buffer: a move takes at most 11
    if (mode != kPropExternal && B.H.ravail < 16) refill_draws(B.H);
    if (threadIdx.x == 0) {
      MoveCtx &mc = B.mc;
      mc.rande = -1.0;
      mc.estep = 0.0;
      mc.overlap = 0;
      mc.accepted = 0;
      mc.surf_new = mc.surf_old = 0;
      B.flags[5] = 0;
      B.flags[6] = 0;
      if (mode == kPropMC) {
        select_move(B, CA, chain);
      } else if (mode == kPropInsert) {
        mc.kind = 1;
        mc.g = g_forced;
        mc.ns = B.S.g[g_forced].ns;
        mc.npos = 1;
        mc.slot = -1;
        mc.choice = 0;
        DrawCursor dc(B.H);
        for (int i = 0; i < 7; ++i) B.draws[i] = dc.next();
        dc.done();
      } else {  // external: kind, g, choice, positions or a,b,c,q given in mc
        mc.ns = B.S.g[mc.g].ns;
        mc.slot = -1;
        mc.npos = mc.kind >= 3 ? 2 : 1;
        if (mc.kind >= 3) {
          B.geo[0] = mc.pos[1][0][0];
          B.geo[1] = mc.pos[1][0][1];
          B.geo[2] = mc.pos[1][0][2];
          B.geo[3] = mc.pos[1][1][0];
          B.geo[4] = mc.pos[1][1][1];
          B.geo[5] = mc.pos[1][1][2];
          B.geo[6] = mc.pos[1][2][0];
          B.draws[3] = 1.0f;  // rotation present
        }
      }
      if (mc.kind == 2 || mc.kind >= 3) {
        int nm = B.H.nummols[mc.g];
        if (mc.choice < 1 || mc.choice > nm) {
          B.H.status |= kStBadChoice;
          mc.kind = 0;
        } else {
          mc.slot = (F32 && CA.resident) ? mc.choice - 1
                                         : CA.ord[((size_t)chain * kMaxG + mc.g) * CA.cap + (mc.choice - 1)];
          if ((unsigned)mc.slot >= (unsigned)CA.cap) {  // a damaged order list
            B.H.status |= kStIndex;
            mc.kind = 0;
          }
        }
      }
    }
    if (threadIdx.x == 0) {
      B.flags[3] = (F32 && mode != kPropExternal) ? 1 : 0;
      B.flags[4] = mode == kPropMC ? 1 : 0;  // delE of other molecule types only if accepted
    }
    __syncwarp();
    if (F32 && mode != kPropExternal) geometry_f32<F32, TRIC>(B, CA, chain);
    else geometry_warp(B, CA, chain, mode);
  }
  __syncthreads();
}

// ------------------------------------------------------------- overlap test
// Any framework or guest site within the overlap distance of any site of
// position 0: the test that lets an insertion or displacement exit before
// the full sums (insertion / guest_energy, mc_moves.f:217-225, 347-355).
// r^2 of one work item of the FP32 overlap test over 27 neighbour cells:
// a site position as a hi/lo pair, neighbour cell c (0..26) of the cell
// holding it and padded slot j of that cell (an empty slot lies far away).
__device__ __forceinline__ float overlap_r2_27(const SysDev &S, const float *ph, const float *pl, int c,
                                               int j) {
  const int lp = S.cpad_log2;
  const int o3[3] = {c / 9 - 1, (c / 3) % 3 - 1, c % 3 - 1};
  int im[3], iw[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    int ic = (int)floorf(ph[d] * S.rcszf[d]) + o3[d];
    int k = 0;
    if (ic < 0) k = -1;
    else if (ic >= S.nc[d]) k = 1;
    if (ic - k * S.nc[d] < 0 || ic - k * S.nc[d] >= S.nc[d]) k = image_of(ic, S.nc[d]);
    im[d] = k;
    iw[d] = ic - k * S.nc[d];
  }
  const size_t a = ((size_t)((iw[0] * S.nc[1] + iw[1]) * S.nc[2] + iw[2]) << lp) + j;
  const float4 H = __ldg(S.cpad_hi + a), L = __ldg(S.cpad_lo + a);
  float ah[3] = {H.x, H.y, H.z}, al[3] = {L.x, L.y, L.z};
  float r2 = 0.f;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (im[d] != 0) {
      float h, e;
      two_sum_f(ah[d], float(im[d]) * S.boxh[d], h, e);
      ah[d] = h;
      al[d] = al[d] + (e + float(im[d]) * S.boxl[d]);
    }
    float dd = (ph[d] - ah[d]) + (pl[d] - al[d]);
    r2 = fmaf(dd, dd, r2);
  }
  return r2;
}

// The FP32 overlap test takes 27 neighbour cells (cells at least the
// overlap distance wide).
__device__ __forceinline__ bool overlap_27(const SysDev &S) {
  const float mincs = fminf(S.cszf[0], fminf(S.cszf[1], S.cszf[2]));
  return S.use_cells && mincs >= sqrtf(S.overlap_sqf) + 0.01f;
}

template <bool F32, bool TRIC>
__device__ int overlap_check(BlockShared<F32> &B, const ChainArrays &CA, int chain) {
  const SysDev &S = B.S;
  const MoveCtx &mc = B.mc;
  const EvalSmem<F32> &ev = B.ev;
  int ns = mc.ns;
  int hit = 0;
  if (S.use_cells) {
    int nrad = 1;
    float mincs = fminf(S.cszf[0], fminf(S.cszf[1], S.cszf[2]));
    float ov = sqrtf(S.overlap_sqf) + 0.01f;
    while (nrad * mincs < ov && nrad < 4) ++nrad;
    int span = 2 * nrad + 1;
    int per_site = span * span * span;
    if (F32 && nrad == 1) {
      // 27 neighbour cells per site, every padded slot of each cell one
      // work item: a single round of independent loads
      const int lp = S.cpad_log2;
      const int nitem = (ns * 27) << lp;
      for (int t = threadIdx.x; t < nitem && !hit; t += kThreads) {
        const int j = t & ((1 << lp) - 1);
        const int sc = t >> lp;
        const int s = sc / 27, c = sc - 27 * s;
        if (overlap_r2_27(S, ev.phi[0][s], ev.plo[0][s], c, j) < S.overlap_sqf) hit = 1;
      }
    } else
    for (int t = threadIdx.x; t < ns * per_site && !hit; t += kThreads) {
      int s = t / per_site, c = t % per_site;
      int o3[3] = {c / (span * span) - nrad, (c / span) % span - nrad, c % span - nrad};
      int im[3], iw[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        int ic = (int)floorf(ev.phi[0][s][d] * S.rcszf[d]) + o3[d];
        im[d] = image_of(ic, S.nc[d]);
        iw[d] = ic - im[d] * S.nc[d];
      }
      int cell = (iw[0] * S.nc[1] + iw[1]) * S.nc[2] + iw[2];
      int a0 = __ldg(S.cell_start + cell), a1 = __ldg(S.cell_start + cell + 1);
      for (int a = a0; a < a1; ++a) {
        if constexpr (F32) {
          float4 H = __ldg(S.fwhi + a), L = __ldg(S.fwlo + a);
          float ah[3] = {H.x, H.y, H.z}, al[3] = {L.x, L.y, L.z};
          float r2 = 0.f;
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            if (im[d] != 0) {
              float h, e;
              two_sum_f(ah[d], float(im[d]) * S.boxh[d], h, e);
              ah[d] = h;
              al[d] = al[d] + (e + float(im[d]) * S.boxl[d]);
            }
            float dd = (ev.phi[0][s][d] - ah[d]) + (ev.plo[0][s][d] - al[d]);
            r2 = fmaf(dd, dd, r2);
          }
          if (r2 < S.overlap_sqf) hit = 1;
        } else {
          double4 A = S.fw64[a];
          double dx = ev.p64[0][s][0] - (A.x + im[0] * S.box[0]);
          double dy = ev.p64[0][s][1] - (A.y + im[1] * S.box[1]);
          double dz = ev.p64[0][s][2] - (A.z + im[2] * S.box[2]);
          if (dx * dx + dy * dy + dz * dz < S.overlap_sq) hit = 1;
        }
      }
    }
  } else if (F32 && TRIC) {  // parallelepiped cell, FP32 path: every framework atom
    for (int t = threadIdx.x; t < ns * S.nfw && !hit; t += kThreads) {
      const int s = t / S.nfw, a = t % S.nfw;
      const float4 H = __ldg(S.fwhi + a), L = __ldg(S.fwlo + a);
      const float ah[3] = {H.x, H.y, H.z}, al[3] = {L.x, L.y, L.z};
      if (mi_tric_r2(S, ev.phi[0][s], ev.plo[0][s], ah, al) < S.overlap_sqf) hit = 1;
    }
  } else {
    for (int t = threadIdx.x; t < ns * S.nfw && !hit; t += kThreads) {
      int s = t / S.nfw, a = t % S.nfw;
      const double *p = ev.p64[0][s];
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
  if (F32 && CA.resident) {  // one guest type, resident in shared memory
    const GuestType &G2 = S.g[0];
    const int n2 = B.H.nummols[0], ns2 = G2.ns;
    const float pre = sqrtf(S.overlap_sqf) + 2.0f * (float)G.rmax + 2.0f * (float)G2.rmax + 0.01f;
    const float pre2 = pre * pre;
    for (int i = threadIdx.x; i < n2 && !hit; i += kThreads) {
      if (i == mc.slot) continue;
      const float4 q0 = B.grh[i * ns2];
      float dx = ev.phi[0][0][0] - q0.x, dy = ev.phi[0][0][1] - q0.y, dz = ev.phi[0][0][2] - q0.z;
      dx -= S.boxh[0] * rint_image(dx * S.rboxf[0]);
      dy -= S.boxh[1] * rint_image(dy * S.rboxf[1]);
      dz -= S.boxh[2] * rint_image(dz * S.rboxf[2]);
      if (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) > pre2) continue;
      for (int b = 0; b < ns2; ++b) {
        const float4 qh = B.grh[i * ns2 + b], ql = B.grl[i * ns2 + b];
        for (int s = 0; s < ns; ++s) {
          float ex = mi_diff32(ev.phi[0][s][0], ev.plo[0][s][0], qh.x, ql.x, S.boxh[0], S.boxl[0], S.rboxf[0]);
          float ey = mi_diff32(ev.phi[0][s][1], ev.plo[0][s][1], qh.y, ql.y, S.boxh[1], S.boxl[1], S.rboxf[1]);
          float ez = mi_diff32(ev.phi[0][s][2], ev.plo[0][s][2], qh.z, ql.z, S.boxh[2], S.boxl[2], S.rboxf[2]);
          if (fmaf(ex, ex, fmaf(ey, ey, ez * ez)) < S.overlap_sqf) hit = 1;
        }
      }
    }
    return block_or(hit, B.ev.red_i);
  }
  for (int g2 = 0; g2 < S.ntpguest && !hit; ++g2) {
    const GuestType &G2 = S.g[g2];
    int n2 = B.H.nummols[g2];
    const int *ord = CA.ord + ((size_t)chain * kMaxG + g2) * CA.cap;
    float pre = sqrtf(S.overlap_sqf) + 2.0f * (float)G.rmax + 2.0f * (float)G2.rmax + 0.01f;
    if constexpr (F32) {
      const float4 *gh = CA.ghi + ((size_t)chain * kMaxG + g2) * CA.cap * kMaxS;
      const float4 *gl = CA.glo + ((size_t)chain * kMaxG + g2) * CA.cap * kMaxS;
      float pre2 = pre * pre;
      for (int i = threadIdx.x; i < n2 && !hit; i += kThreads) {
        int slot = ord[i];
        if ((unsigned)slot >= (unsigned)CA.cap) {
          atomicOr(&B.flags[0], kStIndex);
          continue;
        }
        if (g2 == mc.g && slot == mc.slot) continue;
        float4 q0 = gh[(size_t)slot * kMaxS];
        float dx = ev.phi[0][0][0] - q0.x, dy = ev.phi[0][0][1] - q0.y, dz = ev.phi[0][0][2] - q0.z;
        if (!TRIC || S.use_cells) {
          dx -= S.boxh[0] * rint_image(dx * S.rboxf[0]);
          dy -= S.boxh[1] * rint_image(dy * S.rboxf[1]);
          dz -= S.boxh[2] * rint_image(dz * S.rboxf[2]);
          if (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) > pre2) continue;
        } else if (tric_r2_f32(S, dx, dy, dz) > pre2) {
          continue;
        }
        for (int b = 0; b < G2.ns; ++b) {
          float4 qh = gh[(size_t)slot * kMaxS + b], ql = gl[(size_t)slot * kMaxS + b];
          for (int s = 0; s < ns; ++s) {
            float r2;
            if (!TRIC || S.use_cells) {
              float ex = mi_diff32(ev.phi[0][s][0], ev.plo[0][s][0], qh.x, ql.x, S.boxh[0], S.boxl[0], S.rboxf[0]);
              float ey = mi_diff32(ev.phi[0][s][1], ev.plo[0][s][1], qh.y, ql.y, S.boxh[1], S.boxl[1], S.rboxf[1]);
              float ez = mi_diff32(ev.phi[0][s][2], ev.plo[0][s][2], qh.z, ql.z, S.boxh[2], S.boxl[2], S.rboxf[2]);
              r2 = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
            } else {
              const float qa[3] = {qh.x, qh.y, qh.z}, qb[3] = {ql.x, ql.y, ql.z};
              r2 = mi_tric_r2(S, ev.phi[0][s], ev.plo[0][s], qa, qb);
            }
            if (r2 < S.overlap_sqf) hit = 1;
          }
        }
      }
    } else {
      for (int i = threadIdx.x; i < n2 && !hit; i += kThreads) {
        int slot = ord[i];
        if ((unsigned)slot >= (unsigned)CA.cap) {
          atomicOr(&B.flags[0], kStIndex);
          continue;
        }
        if (g2 == mc.g && slot == mc.slot) continue;
        const double *q = CA.gpos + gslot_base(CA, chain, g2, slot) * 3;
        if (S.use_cells) {
          double dx = ev.p64[0][0][0] - q[0], dy = ev.p64[0][0][1] - q[1], dz = ev.p64[0][0][2] - q[2];
          dx -= S.box[0] * round(S.rbox[0] * dx);
          dy -= S.box[1] * round(S.rbox[1] * dy);
          dz -= S.box[2] * round(S.rbox[2] * dz);
          if (dx * dx + dy * dy + dz * dz > (double)pre * (double)pre) continue;
        }
        for (int b = 0; b < G2.ns; ++b)
          for (int s = 0; s < ns; ++s) {
            double ex = ev.p64[0][s][0] - q[3 * b], ey = ev.p64[0][s][1] - q[3 * b + 1],
                   ez = ev.p64[0][s][2] - q[3 * b + 2];
            if (S.use_cells) {
              ex -= S.box[0] * round(S.rbox[0] * ex);
              ey -= S.box[1] * round(S.rbox[1] * ey);
              ez -= S.box[2] * round(S.rbox[2] * ez);
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
  }
  return block_or(hit, B.ev.red_i);
}

// ----------------------------------------------------------------- k-space
// One pass over the k-vectors for npos positions (ewald1_guest, ewald.f:
// 151-315): s(k) of position 0 goes to the snew scratch and of position 1 to
// sold; energies and mixing terms accumulate in acc.
template <bool F32, int GN, int NS>
__device__ __forceinline__ void kspace(BlockShared<F32> &B, const ChainArrays &CA, int chain,
                                       bool exist0, PosAcc<F32, GN> &acc0, PosAcc<F32, GN> &acc1,
                                       int &st) {
  const SysDev &S = B.S;
  const MoveCtx &mc = B.mc;
  const GuestType &G = S.g[mc.g];
  const int ns = NS > 0 ? NS : mc.ns, npos = mc.npos, mol = G.mol, NG = S.ntpguest;
  const bool disp = npos == 2;
  if constexpr (!F32) {
    double2 *snew = CA.snew + (size_t)chain * CA.nkmax;
    double2 *sold = CA.sold + (size_t)chain * CA.nkmax;
    const double2 *skg = CA.sk + (size_t)chain * kMaxG * CA.nkmax;
    double e[2] = {0.0, 0.0}, mfw[2] = {0.0, 0.0}, mg[2][GN];
#pragma unroll
    for (int g2 = 0; g2 < GN; ++g2) mg[0][g2] = mg[1][g2] = 0.0;
    int kb, ke;  // this CTA's share of the k-vectors
    share_of(S.nk, B.ev.rank, B.ev.csize, kb, ke);
    for (int k = kb + threadIdx.x; k < ke; k += kThreads) {
      int4 lmn = __ldg(S.klmn + k);
      int am = abs(lmn.y), an = abs(lmn.z);
      bool cm = lmn.y < 0, cn = lmn.z < 0;
      double akk = __ldg(S.akk + k);
      double2 sfw = __ldg(S.skfw + k);
      double2 stot = sfw;
      double2 sgt[GN];
#pragma unroll
      for (int g2 = 0; g2 < GN; ++g2) {
        if (g2 < NG) {
          sgt[g2] = skg[(size_t)g2 * CA.nkmax + k];
          stot.x += sgt[g2].x;
          stot.y += sgt[g2].y;
        }
      }
      double2 sp[2] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
#pragma unroll
      for (int p = 0; p < 2; ++p) {
        if (p >= npos) break;
        double2 a = make_double2(0.0, 0.0);
        for (int s = 0; s < ns; ++s) {
          double2 ex = B.ev.pw64[p][s][0][lmn.x];
          double2 ey = B.ev.pw64[p][s][1][am];
          double2 ez = B.ev.pw64[p][s][2][an];
          if (cm) ey.y = -ey.y;
          if (cn) ez.y = -ez.y;
          double2 t = cmul(cmul(ex, ey), ez);
          a.x += G.q[s] * t.x;
          a.y += G.q[s] * t.y;
        }
        sp[p] = a;
      }
#pragma unroll
      for (int p = 0; p < 2; ++p) {
        if (p >= npos) break;
        double2 su = stot;
        if (disp && p == 0) {  // the new position sees S - s_old (gcmc.f:2862-2871)
          su.x -= sp[1].x;
          su.y -= sp[1].y;
        }
        bool exist = disp ? (p == 1) : exist0;
        double sumsqd = sp[p].x * sp[p].x + sp[p].y * sp[p].y;
        double mixterm = 2.0 * sp[p].x * su.x + 2.0 * sp[p].y * su.y;
        if (exist) mixterm = -1.0 * mixterm;
        e[p] += akk * (mixterm + sumsqd);
        double f2 = 2.0 * akk;
        mfw[p] += f2 * (sp[p].x * sfw.x + sp[p].y * sfw.y);
#pragma unroll
        for (int g2 = 0; g2 < GN; ++g2)
          if (g2 < NG && S.g[g2].mol != mol) mg[p][g2] += f2 * (sp[p].x * sgt[g2].x + sp[p].y * sgt[g2].y);
      }
      snew[k] = sp[0];
      if (disp) sold[k] = sp[1];
    }
#pragma unroll
    for (int p = 0; p < 2; ++p) {
      PosAcc<F32, GN> &A = p == 0 ? acc0 : acc1;
      A.recip.add(e[p]);
      A.mixfw.add(mfw[p]);
#pragma unroll
      for (int g2 = 0; g2 < GN; ++g2) A.mixg[g2].add(mg[p][g2]);
    }
  } else {
    // Two k-vectors per thread in flight.  e^{i k.r} of a site is the (l, m)
    // table entry times e^{i 2 pi n s_z} (conjugated for n < 0); without the
    // table (large kmax) it is X_l Y_m Z_n from the power tables.
    // the guest S(k) of each type in its current buffer; the moving type's
    // updated S(k) (as commit would form it) goes to its other buffer
    auto skcur = [&](int g2) -> const float4 * {
      return (B.H.skb[g2] ? CA.skdf2 : CA.skdf) + ((size_t)chain * kMaxG + g2) * CA.nkmax;
    };
    float4 *sknext = (B.H.skb[mc.g] ? CA.skdf : CA.skdf2) + ((size_t)chain * kMaxG + mc.g) * CA.nkmax;
    const int kind = mc.kind;
    const int k2 = S.kmax[1], w = 2 * k2 + 1, nlm = (S.kmax[0] + 1) * w;
    const bool tab = B.ev.tabpos * ns * nlm <= kPlmMax;  // independent of npos (EvalSmem::tabpos)
    unsigned mixmask = 0;  // guest types of another molecule type (mixing terms)
    for (int g2 = 0; g2 < NG && g2 < GN; ++g2)
      if (S.g[g2].mol != mol) mixmask |= 1u << g2;
    float e[2] = {0.f, 0.f}, mfw[2] = {0.f, 0.f}, mg[2][GN];
#pragma unroll
    for (int g2 = 0; g2 < GN; ++g2) mg[0][g2] = mg[1][g2] = 0.f;
    int cnt = 0;
    constexpr int U = 2;
    int kb, ke;  // this CTA's share of the k-vectors
    share_of(S.nk, B.ev.rank, B.ev.csize, kb, ke);
    for (int k0 = kb + threadIdx.x; k0 < ke; k0 += U * kThreads) {
      unsigned pk[U];
      float akk[U];
      float4 fw[U], st4[U], vg[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int k = k0 + u * kThreads;
        pk[u] = 0u;
        akk[u] = 0.f;
        fw[u] = st4[u] = vg[u] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (k < ke) {
          pk[u] = __ldg(S.kpk + k);
          akk[u] = __ldg(S.akk32 + k);
          fw[u] = __ldg(S.skfw_df + k);
          st4[u] = fw[u];
          for (int g2 = 0; g2 < NG; ++g2) {
            const float4 v = skcur(g2)[k];
            if (g2 == mc.g) vg[u] = v;
            st4[u].x += v.x;
            st4[u].y += v.y;
            st4[u].z += v.z;
            st4[u].w += v.w;
          }
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int k = k0 + u * kThreads;
        if (k >= ke) continue;
        const int lm = (int)(pk[u] & 0xffffu), nz = (int)(pk[u] >> 16) - 128;
        const int an = abs(nz);
        const bool cn = nz < 0;
        int lx = 0, am = 0;
        bool cm = false;
        if (!tab) {
          lx = lm / w;
          const int mm = lm - lx * w - k2;
          am = abs(mm);
          cm = mm < 0;
        }
        const float2 stot = make_float2(st4[u].x + st4[u].z, st4[u].y + st4[u].w);
        const float2 sfw = make_float2(fw[u].x + fw[u].z, fw[u].y + fw[u].w);
        float2 sp[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
        for (int p = 0; p < 2; ++p) {
          if (p >= npos) break;
          float2 a = make_float2(0.f, 0.f);
#pragma unroll
          for (int s = 0; s < (NS > 0 ? NS : ns); ++s) {
            float2 P;
            if (tab) {
              P = B.ev.plm[(p * ns + s) * nlm + lm];
            } else {
              float2 ey = B.ev.pw32[p][s][1][am];
              if (cm) ey.y = -ey.y;
              P = cmul(B.ev.pw32[p][s][0][lx], ey);
            }
            float2 ez = B.ev.pw32[p][s][2][an];
            if (cn) ez.y = -ez.y;
            const float2 tt = cmul(P, ez);
            const float q = B.si[s].qf;
            a.x = fmaf(q, tt.x, a.x);
            a.y = fmaf(q, tt.y, a.y);
          }
          sp[p] = a;
        }
#pragma unroll
        for (int p = 0; p < 2; ++p) {
          if (p >= npos) break;
          float2 su = stot;
          if (disp && p == 0) {  // the new position sees S - s_old (gcmc.f:2862-2871)
            su.x -= sp[1].x;
            su.y -= sp[1].y;
          }
          const bool exist = disp ? (p == 1) : exist0;
          const float sumsqd = fmaf(sp[p].x, sp[p].x, sp[p].y * sp[p].y);
          float mixterm = 2.0f * fmaf(sp[p].x, su.x, sp[p].y * su.y);
          if (exist) mixterm = -mixterm;
          e[p] = fmaf(akk[u], mixterm + sumsqd, e[p]);
          const float f2 = 2.0f * akk[u];
          mfw[p] = fmaf(f2, fmaf(sp[p].x, sfw.x, sp[p].y * sfw.y), mfw[p]);
          if (mixmask) {
#pragma unroll
            for (int g2 = 0; g2 < GN; ++g2)
              if (mixmask & (1u << g2)) {
                const float4 v = skcur(g2)[k];
                mg[p][g2] = fmaf(f2, fmaf(sp[p].x, v.x + v.z, sp[p].y * (v.y + v.w)), mg[p][g2]);
              }
          }
        }
        {  // the S(k) update of accept_move (mc_moves.f:485-622), in hi/lo
          float4 v = vg[u];
          if (kind == 1) {
            df_inc(v.x, v.z, sp[0].x);
            df_inc(v.y, v.w, sp[0].y);
          } else if (kind == 2) {
            df_inc(v.x, v.z, -sp[0].x);
            df_inc(v.y, v.w, -sp[0].y);
          } else {
            df_inc(v.x, v.z, -sp[1].x);
            df_inc(v.y, v.w, -sp[1].y);
            df_inc(v.x, v.z, sp[0].x);
            df_inc(v.y, v.w, sp[0].y);
          }
          sknext[k] = v;
        }
        if (++cnt == 8) {
#pragma unroll
          for (int p = 0; p < 2; ++p) {
            PosAcc<F32, GN> &A = p == 0 ? acc0 : acc1;
            A.recip.add(e[p]);
            A.mixfw.add(mfw[p]);
            e[p] = mfw[p] = 0.f;
#pragma unroll
            for (int g2 = 0; g2 < GN; ++g2) {
              A.mixg[g2].add(mg[p][g2]);
              mg[p][g2] = 0.f;
            }
          }
          cnt = 0;
        }
      }
    }
#pragma unroll
    for (int p = 0; p < 2; ++p) {
      PosAcc<F32, GN> &A = p == 0 ? acc0 : acc1;
      A.recip.add(e[p]);
      A.mixfw.add(mfw[p]);
#pragma unroll
      for (int g2 = 0; g2 < GN; ++g2) A.mixg[g2].add(mg[p][g2]);
    }
  }
}

// Guest-guest terms with the guests resident in shared memory (one guest
// type, molecule order): the terms of scan_guests, without the slot
// indirection and global loads.
template <bool F32, int GN, int NS>
__device__ __forceinline__ void scan_guests_resident(BlockShared<F32> &B, int pos, int ns_rt,
                                                     int self_i, float rmax_self,
                                                     PosAcc<F32, GN> &acc, int &ov, int &sf,
                                                     int &st) {
  const SysDev &S = B.S;
  const EvalSmem<F32> &sm = B.ev;
  const SiteInfo *si = B.si;
  const int ns = NS > 0 ? NS : ns_rt;
  const GuestType &G2 = S.g[0];
  const int n2 = B.H.nummols[0], ns2 = G2.ns;
  const float pre = (float)S.rcut + 2.0f * rmax_self + 2.0f * (float)G2.rmax + 0.01f;
  const float pre2 = pre * pre;
  int i0, i1;
  share_of(n2, sm.rank, sm.csize, i0, i1);
  for (int i = i0 + threadIdx.x; i < i1; i += kThreads) {
    if (i == self_i) continue;
    const float4 q0 = B.grh[i * ns2];
    float dx = sm.phi[pos][0][0] - q0.x, dy = sm.phi[pos][0][1] - q0.y, dz = sm.phi[pos][0][2] - q0.z;
    dx -= S.boxh[0] * rint_image(dx * S.rboxf[0]);
    dy -= S.boxh[1] * rint_image(dy * S.rboxf[1]);
    dz -= S.boxh[2] * rint_image(dz * S.rboxf[2]);
    if (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) > pre2) continue;
    float vdw = 0.f;
#pragma unroll
    for (int b = 0; b < (NS > 0 ? NS : ns2); ++b) {  // the same guest type: ns2 == ns
      const float4 qh = B.grh[i * ns2 + b], ql = B.grl[i * ns2 + b];
      const int tb = G2.type[b];
#pragma unroll
      for (int k = 0; k < (NS > 0 ? NS : ns); ++k) {
        float ex = mi_diff32(sm.phi[pos][k][0], sm.plo[pos][k][0], qh.x, ql.x, S.boxh[0],
                             S.boxl[0], S.rboxf[0]);
        float ey = mi_diff32(sm.phi[pos][k][1], sm.plo[pos][k][1], qh.y, ql.y, S.boxh[1],
                             S.boxl[1], S.rboxf[1]);
        float ez = mi_diff32(sm.phi[pos][k][2], sm.plo[pos][k][2], qh.z, ql.z, S.boxh[2],
                             S.boxl[2], S.rboxf[2]);
        float r2 = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
        const bool near = vdw_is_near(S, si[k], tb, r2);
        pair_term32(S, si[k], qh.w, ql.w, tb, G2.frz[b], r2, acc.e2g[0], vdw, ov, sf, st, near);
        if (near) {
          float dh[3], dl[3];
          mi_diff_df(sm.phi[pos][k][0], sm.plo[pos][k][0], qh.x, ql.x, S.boxh[0], S.boxl[0],
                     S.rboxf[0], dh[0], dl[0]);
          mi_diff_df(sm.phi[pos][k][1], sm.plo[pos][k][1], qh.y, ql.y, S.boxh[1], S.boxl[1],
                     S.rboxf[1], dh[1], dl[1]);
          mi_diff_df(sm.phi[pos][k][2], sm.plo[pos][k][2], qh.z, ql.z, S.boxh[2], S.boxl[2],
                     S.rboxf[2], dh[2], dl[2]);
          acc.vdwg[0].add_df(vdw_near_df(S, si[k], tb, dh, dl, st));
        }
      }
    }
    acc.vdwg[0].add(vdw);
  }
}

// Guest sites of one guest type for the two-stage scan below: in shared
// memory (resident, molecule i in slot i) or in global memory (slot ord[i]).
template <bool F32>
struct ResidentSites {
  const BlockShared<F32> &B;
  int ns;
  __device__ __forceinline__ float4 hi(int i, int b) const { return B.grh[i * ns + b]; }
  __device__ __forceinline__ float4 lo(int i, int b) const { return B.grl[i * ns + b]; }
  __device__ __forceinline__ bool is_self(int i, int self_slot) const { return i == self_slot; }
};
struct GlobalSites {
  const float4 *gh, *gl;
  const int *ord;
  __device__ __forceinline__ float4 hi(int i, int b) const {
    return gh[(size_t)ord[i] * kMaxS + b];
  }
  __device__ __forceinline__ float4 lo(int i, int b) const {
    return gl[(size_t)ord[i] * kMaxS + b];
  }
  __device__ __forceinline__ bool is_self(int i, int self_slot) const { return ord[i] == self_slot; }
};

// Guests of one type, first stage: this CTA's share of the molecules whose
// first site lies within the cutoff plus both molecules' extents of
// position pos, listed in a fixed order (thread, then stride) so that the
// sums that follow do not depend on timing.  Returns false (uniformly)
// when the share is longer than the list; the per-molecule loop then runs.
// self_slot: the moving molecule's slot (-1 for an insertion).
template <bool F32, class Sites>
__device__ __forceinline__ bool list_near_guests(BlockShared<F32> &B, const Sites &gs, int pos,
                                                 int self_slot, float rmax_self) {
  const SysDev &S = B.S;
  EvalSmem<F32> &sm = B.ev;
  const GuestType &G2 = S.g[0];
  const int n2 = B.H.nummols[0];
  int i0, i1;
  share_of(n2, sm.rank, sm.csize, i0, i1);
  if (i1 - i0 > kGList) return false;
  const float pre = (float)S.rcut + 2.0f * rmax_self + 2.0f * (float)G2.rmax + 0.01f;
  const float pre2 = pre * pre;
  int cnt = 0, m0 = 0, m1 = 0;
#pragma unroll
  for (int k = 0; k < kGList / kThreads; ++k) {
    const int i = i0 + threadIdx.x + k * kThreads;
    if (i < i1 && !gs.is_self(i, self_slot)) {
      const float4 q0 = gs.hi(i, 0);
      float dx = sm.phi[pos][0][0] - q0.x, dy = sm.phi[pos][0][1] - q0.y, dz = sm.phi[pos][0][2] - q0.z;
      dx -= S.boxh[0] * rint_image(dx * S.rboxf[0]);
      dy -= S.boxh[1] * rint_image(dy * S.rboxf[1]);
      dz -= S.boxh[2] * rint_image(dz * S.rboxf[2]);
      if (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= pre2) {
        if (cnt == 0) m0 = i;
        else m1 = i;
        ++cnt;
      }
    }
  }
  int excl;
  const int tot = block_scan(cnt, excl, sm.red_i);
  if (cnt > 0) sm.glist[excl] = m0;
  if (cnt > 1) sm.glist[excl + 1] = m1;
  if (threadIdx.x == 0) sm.gcount = tot;
  __syncthreads();
  return true;
}

// Second stage: one site pair (molecule of the list, its site b, the
// position's site k) per work item, so a near molecule's ns^2 pair terms
// spread over ns^2 threads.  One guest type (the moving one: ns2 == ns).
template <bool F32, int GN, int NS, class Sites>
__device__ __forceinline__ void scan_guest_pairs(BlockShared<F32> &B, const Sites &gs, int pos,
                                                 int ns_rt, PosAcc<F32, GN> &acc, int &ov, int &sf,
                                                 int &st) {
  const SysDev &S = B.S;
  const EvalSmem<F32> &sm = B.ev;
  const SiteInfo *si = B.si;
  const int ns = NS > 0 ? NS : ns_rt;
  const GuestType &G2 = S.g[0];
  const int per = ns * ns;
  const int nitem = sm.gcount * per;
  for (int t = threadIdx.x; t < nitem; t += kThreads) {
    const int j = t / per, r = t - j * per;
    const int b = r / ns, k = r - b * ns;
    const int i = sm.glist[j];
    const float4 qh = gs.hi(i, b), ql = gs.lo(i, b);
    const int tb = G2.type[b];
    const float ex = mi_diff32(sm.phi[pos][k][0], sm.plo[pos][k][0], qh.x, ql.x, S.boxh[0],
                               S.boxl[0], S.rboxf[0]);
    const float ey = mi_diff32(sm.phi[pos][k][1], sm.plo[pos][k][1], qh.y, ql.y, S.boxh[1],
                               S.boxl[1], S.rboxf[1]);
    const float ez = mi_diff32(sm.phi[pos][k][2], sm.plo[pos][k][2], qh.z, ql.z, S.boxh[2],
                               S.boxl[2], S.rboxf[2]);
    const float r2 = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
    const bool near = vdw_is_near(S, si[k], tb, r2);
    float vdw = 0.f;
    pair_term32(S, si[k], qh.w, ql.w, tb, G2.frz[b], r2, acc.e2g[0], vdw, ov, sf, st, near);
    if (near) {
      float dh[3], dl[3];
      mi_diff_df(sm.phi[pos][k][0], sm.plo[pos][k][0], qh.x, ql.x, S.boxh[0], S.boxl[0],
                 S.rboxf[0], dh[0], dl[0]);
      mi_diff_df(sm.phi[pos][k][1], sm.plo[pos][k][1], qh.y, ql.y, S.boxh[1], S.boxl[1],
                 S.rboxf[1], dh[1], dl[1]);
      mi_diff_df(sm.phi[pos][k][2], sm.plo[pos][k][2], qh.z, ql.z, S.boxh[2], S.boxl[2],
                 S.rboxf[2], dh[2], dl[2]);
      acc.vdwg[0].add_df(vdw_near_df(S, si[k], tb, dh, dl, st));
    }
    acc.vdwg[0].add(vdw);
  }
}

// delE(m) against every molecule type m other than the moving one, from
// the block totals in ev.out (thread 0).  In the main loop it is needed only
// to update energy(m) of an accepted move, so it runs after the decision.
template <bool F32, int GN>
__device__ void other_mol_delE(BlockShared<F32> &B, int kind, int g, int npos, double *delE) {
  const SysDev &S = B.S;
  const GuestType &G = S.g[g];
  constexpr int nper = PosAcc<F32, GN>::kN;
  const double *R = B.ev.out;
  const int NG = S.ntpguest, mol = G.mol;
  const double eu = S.rengunit;
  auto pair_terms = [&](int p, int m, double delrc_m) {
    const double *r = R + p * nper;
    bool exist = (npos == 2) ? (p == 1) : (kind == 2);
    double qfm = G.qfm * B.H.chgsum_mol[m];
    if (exist) qfm = -qfm;
    double e1 = 0.0, e2m = 0.0, vdm = 0.0;
    if (m == S.fw_mol) {
      e1 = S.krecip * r[3] + qfm;
      e2m = r[0];
      vdm = r[1];
    } else {
      e1 = qfm;
      for (int g2 = 0; g2 < NG; ++g2)
        if (S.g[g2].mol == m) {
          e1 += S.krecip * r[4 + 2 * GN + g2];
          e2m += r[4 + g2];
          vdm += r[4 + GN + g2];
        }
    }
    return e1 + e2m + vdm + delrc_m;
  };
  if (kind == 1 || kind == 2) {
    const bool del = kind == 2;
    for (int m = 1; m <= S.maxmls; ++m) {
      if (m == mol) continue;
      double dm = 0.0;  // delrc_mol(loc2(mol,m)), vdw_terms.f:743-761
      if (m == S.fw_mol) dm = G.lrcA - G.lrcC;
      else
        for (int g2 = 0; g2 < NG; ++g2)
          if (S.g[g2].mol == m) dm = double(B.H.nummols[g2]) * G.lrcB[g2];
      const double t = pair_terms(0, m, dm) * eu;
      delE[m] = del ? -t : t;
    }
  } else {
    for (int m = 1; m <= S.maxmls; ++m)
      if (m != mol) delE[m] = (pair_terms(0, m, 0.0) - pair_terms(1, m, 0.0)) * eu;
  }
}

// --------------------------------------------------------------- evaluate
// Evaluate the proposed move; fills mc.estep, mc.delE and the flags.
// Returns 1 if a full evaluation ran (no overlap exit).
template <bool F32, int GN, int NS>
__device__ int evaluate(BlockShared<F32> &B, const ChainArrays &CA, int chain, int &st) {
  const SysDev &S = B.S;
  MoveCtx &mc = B.mc;
  const GuestType &G = S.g[mc.g];
  const int ns = NS > 0 ? NS : mc.ns, npos = mc.npos, NG = S.ntpguest;
  if (!B.flags[3]) {  // positions from FP64 geometry: site constants, FP32 pairs, bounds
    if (threadIdx.x < ns) {
      int s = threadIdx.x;
      B.si[s].q = G.q[s];
      B.si[s].chgea = G.chgea[s];
      B.si[s].chgeaf = G.chgeaf[s];
      B.si[s].chgeaf_lo = G.chgeaf_lo[s];
      B.si[s].qf = (float)G.q[s];
      B.si[s].type = G.type[s];
      B.si[s].prow = G.prow[s];
      B.si[s].psig2 = G.psig2[s];
    }
    if (threadIdx.x == 0) B.si_g = mc.g;
    if (threadIdx.x >= 32 && threadIdx.x < 32 + 2 * kMaxS * 3) {
      int t = threadIdx.x - 32;
      int p = t / (kMaxS * 3), s = (t / 3) % kMaxS, d = t % 3;
      if (p < npos && s < ns) {
        double v = mc.pos[p][s][d];
        B.ev.p64[p][s][d] = v;
        float h = (float)v;
        B.ev.phi[p][s][d] = h;
        B.ev.plo[p][s][d] = (float)(v - (double)h);
      }
    }
    __syncthreads();
    if (threadIdx.x < 32) position_bounds(B, threadIdx.x);  // conservative (FP32)
    __syncthreads();
  }
  if (B.flags[7]) {  // positions out of range: no evaluation, reported
    if (threadIdx.x == 0) {
      mc.overlap = 1;
      mc.estep = 0.0;
    }
    st |= kStIndex;
    __syncthreads();
    return 0;
  }
  if (mc.kind == 1 || mc.kind >= 3) {
    if (!B.flags[6]) {  // flags[6]: a speculative round found this position clear already
      const int hit = overlap_check<F32, kTricOk<F32, GN>>(B, CA, chain);
      FMC_PHASE(B, 1);
      if (hit) {
        if (threadIdx.x == 0) mc.overlap = 1;
        __syncthreads();
        return 0;
      }
    }
    if constexpr (F32) {
      // FP32 first-pass geometry: warp 0 refines it; the positions are
      // next read after build_segments' barriers
      if (B.flags[3] && threadIdx.x < 32) refine_geometry<F32, kTricOk<F32, GN>>(B, CA);
    }
  }
  PosAcc<F32, GN> acc0, acc1;
  acc0.zero();
  acc1.zero();
  int sf0 = 0, sf1 = 0, ovd = 0;
  auto scan_position = [&](int p, PosAcc<F32, GN> &A, int &sfp) {
    build_segments<F32>(S, B.ev, B.ev.cen[p], (float)S.rcut + B.ev.rmx[p] + 1e-3f, st);
    // one guest type on the FP32 path: near molecules listed, then one
    // site pair per work item (resident or global guests alike)
    bool listed = false;
    const ResidentSites<F32> rs{B, ns};
    const GlobalSites gsites{CA.ghi + (size_t)chain * kMaxG * CA.cap * kMaxS,
                             CA.glo + (size_t)chain * kMaxG * CA.cap * kMaxS,
                             CA.ord + (size_t)chain * kMaxG * CA.cap};
    if constexpr (F32 && GN == 1) {
      if (CA.resident) listed = list_near_guests(B, rs, p, mc.slot, B.ev.rmx[p]);
      else if (S.use_cells) listed = list_near_guests(B, gsites, p, mc.slot, B.ev.rmx[p]);
    }
    FMC_PHASE_SYNC(B, 2);
    scan_framework<F32, NS, kTricOk<F32, GN>>(S, B.ev, p, ns, B.si, A, ovd, sfp, st);
    bool done = false;
    if constexpr (F32 && GN == 1) {
      if (listed) {
        if (CA.resident) scan_guest_pairs<F32, GN, NS>(B, rs, p, ns, A, ovd, sfp, st);
        else scan_guest_pairs<F32, GN, NS>(B, gsites, p, ns, A, ovd, sfp, st);
        done = true;
      }
    }
    if constexpr (F32) {
      if (!done && CA.resident) {
        scan_guests_resident<F32, GN, NS>(B, p, ns, mc.slot, B.ev.rmx[p], A, ovd, sfp, st);
        done = true;
      }
    }
    if (!done)
      scan_guests<F32, GN, NS>(S, B.H, CA, chain, B.ev, p, ns, mc.g, mc.slot, B.ev.rmx[p], B.si, A,
                               ovd, sfp, st);
    __syncthreads();
    FMC_PHASE(B, 3);
  };
  scan_position(0, acc0, sf0);
  if (npos == 2) scan_position(1, acc1, sf1);
  build_powers<F32, kTricOk<F32, GN>>(S, B.ev, npos, ns);
  __syncthreads();
  FMC_PHASE(B, 4);
  kspace<F32, GN, NS>(B, CA, chain, mc.kind == 2, acc0, acc1, st);
  FMC_PHASE_SYNC(B, 5);
  // block totals: out[p * nper + j], j = e2fw, vdwfw, recip, mixfw,
  // e2g[GN], vdwg[GN], mixg[GN]
  constexpr int nper = PosAcc<F32, GN>::kN;
  const int sfl = block_reduce_pos<F32, GN>(acc0, acc1, npos, NG, B.ev.red, B.ev.out,
                                            (sf0 ? 1 : 0) | (sf1 ? 2 : 0), B.ev.red_i);
  int sfa = sfl & 1;
  int sfb = (sfl >> 1) & 1;
  FMC_PHASE(B, 6);
  if (B.ev.csize > 1) {  // totals over the cluster
    if (threadIdx.x == 0) {
      B.ev.out[2 * nper] = sfa;
      B.ev.out[2 * nper + 1] = sfb;
    }
    cluster_exchange(B, 2 * nper + 2, st);
    sfa = B.ev.out[2 * nper] > 0.5;
    sfb = B.ev.out[2 * nper + 1] > 0.5;
    FMC_PHASE(B, 7);
  }
  if (threadIdx.x == 0) {
    const double *R = B.ev.out;
    mc.surf_new = sfa;
    mc.surf_old = sfb;
    const int mol = G.mol;
    const double sumchg = B.H.sumchg, eu = S.rengunit, e3 = G.ewald3en;
    double ewld1[2], e2[2], vd[2];
    for (int p = 0; p < npos; ++p) {
      const double *r = R + p * nper;
      bool exist = (npos == 2) ? (p == 1) : (mc.kind == 2);
      double sic = exist ? -G.engsic0 : G.engsic0;
      double qfix = G.qfa * sumchg + G.qfb;
      if (exist) qfix = -qfix;
      ewld1[p] = S.krecip * r[2] + sic + qfix;
      e2[p] = r[0];
      vd[p] = r[1];
      for (int g2 = 0; g2 < NG; ++g2) {
        e2[p] += r[4 + g2];
        vd[p] += r[4 + GN + g2];
      }
    }
    for (int m = 0; m <= kMaxM; ++m) mc.delE[m] = 0.0;
    if (mc.kind == 1 || mc.kind == 2) {
      bool del = mc.kind == 2;
      double delrc = lrc_delta(S, B.H, mc.g, del);
      mc.delrc = delrc;
      if (!del) mc.estep = (ewld1[0] + e2[0] - e3 + vd[0] + delrc) * eu;
      else mc.estep = (-ewld1[0] + e2[0] + vd[0] - e3) * eu - delrc * eu;
      mc.delE[mol] = del ? -mc.estep : mc.estep;
    } else {
      double enginit = (-ewld1[1] + e2[1] + vd[1] - e3) * eu;
      double enew = (ewld1[0] + e2[0] + vd[0] - e3) * eu;
      mc.estep = enew - enginit;
      mc.delrc = 0.0;
      mc.delE[mol] = mc.estep;
    }
    if (!B.flags[4]) other_mol_delE<F32, GN>(B, mc.kind, mc.g, mc.npos, mc.delE);
    mc.parts[0] = ewld1[0];
    mc.parts[1] = e2[0];
    mc.parts[2] = vd[0];
    mc.parts[3] = mc.delrc;
    mc.chgtmp = G.chgtmp;
    if (!isfinite(mc.estep)) st |= kStNonFinite;
  }
  __syncthreads();
  FMC_PHASE(B, 8);
  return 1;
}

// evaluate with the site loops unrolled for three-site guests (FP32 path).
template <bool F32, int GN>
__device__ __forceinline__ int evaluate_any(BlockShared<F32> &B, const ChainArrays &CA, int chain,
                                            int &st) {
  if constexpr (F32) {
    if (B.mc.ns == 3) return evaluate<F32, GN, 3>(B, CA, chain, st);
  }
  return evaluate<F32, GN, 0>(B, CA, chain, st);
}

// The same, called rather than inlined: for the moves and modes that run
// seldom (pre-loading, restart loading, swap and switch halves), so that the
// kernel holds one more copy of the evaluation instead of one per call site.
template <bool F32, int GN>
__device__ __noinline__ int evaluate_rare(BlockShared<F32> &B, const ChainArrays &CA, int chain,
                                          int &st) {
  return evaluate_any<F32, GN>(B, CA, chain, st);
}

// ----------------------------------------------------------------- decide
// Thread 0.  `draw`: take the Metropolis number from the chain's generator.
template <bool F32>
__device__ void decide(BlockShared<F32> &B, bool draw) {
  MoveCtx &mc = B.mc;
  ChainHdr &H = B.H;
  if (mc.kind == 0) {
    mc.accepted = B.flags[5] ? H.last_accepted : 0;
    return;
  }
  if (mc.kind == 1) {
    if (mc.overlap) {
      mc.accepted = 0;
      return;
    }
    if (draw) mc.rande = (double)draw_f(H);
    mc.accepted = energy_eval<F32>(B.S, H, mc.g, mc.estep, mc.rande, 1);
  } else if (mc.kind == 2) {
    if (draw) mc.rande = (double)draw_f(H);
    mc.accepted = energy_eval<F32>(B.S, H, mc.g, -mc.estep, mc.rande, 2);
  } else {
    if (mc.overlap) {
      mc.accepted = 0;
      return;
    }
    if (mc.estep < 0.0) {
      mc.accepted = 1;
      if (draw) mc.rande = -1.0;
    } else {
      if (draw) mc.rande = (double)draw_f(H);
      mc.accepted = energy_eval<F32>(B.S, H, mc.g, mc.estep, mc.rande, mc.kind);
    }
  }
}


// FP32 path: the production sums of H.pend moves that all saw the current
// state (the reference adds one move at a time, gcmc.f:1050-1075; here the
// run is added at once when the state changes or a window ends).
__device__ inline void flush_stats(const SysDev &S, ChainHdr &H, int g_old = -1, int n_old = 0) {
  if (H.pend == 0) return;
  const double n = (double)H.pend;
  for (int i = 0; i < S.ntpguest; ++i) {
    int m = S.g[i].mol;
    double dm = double((float)(i == g_old ? n_old : H.nummols[i]));
    double e = H.energy[m];
    double sm = double((float)H.surfacemols[m]);
    H.chainstats[i][0] += n * dm;
    H.chainstats[i][1] += n * e;
    H.chainstats[i][2] += n * (e * dm);
    H.chainstats[i][3] += n * (dm * dm);
    H.chainstats[i][4] += n * (e * e);
    H.chainstats[i][5] += n * sm;
  }
  H.pend = 0;
}

// ----------------------------------------------------------------- commit
// accept_move (mc_moves.f:485-621) for the evaluated move, if accepted.
// The FP64 state updates of accept_move (mc_moves.f:485-622) for one
// accepted move of guest type g: production sums of the moves that saw the
// old state (FP32 path, n_old = the type's count before the move), energies,
// charges and the surface tally.
template <bool F32>
__device__ inline void bookkeep(const SysDev &S, ChainHdr &H, int g, int n_old, int kind,
                                const double *delE, double chgtmp, int surf_new, int surf_old) {
  if constexpr (F32) flush_stats(S, H, g, n_old);  // the pending moves saw the old state
  for (int m = 1; m <= S.maxmls; ++m) H.energy[m] += delE[m];
  const int mol = S.g[g].mol;
  if (kind == 1 || kind == 2) {
    const int sg = kind == 1 ? 1 : -1;
    H.chgsum_mol[mol] += sg * chgtmp;
    H.sumchg += sg * chgtmp;
    if (surf_new) H.surfacemols[mol] += sg;
  } else {
    // surface molecule tally of a displacement (gcmc.f:1900-1906)
    if (surf_old && !surf_new) {
      H.surfacemols[mol] -= 1;
      if (H.surfacemols[mol] < 0) H.surfacemols[mol] = 0;
    } else if (!surf_old && surf_new) {
      H.surfacemols[mol] += 1;
    }
  }
}

// defer: the main loop's commit leaves bookkeep() to run_deferred (thread
// 32, during the next proposal); the integer state the next move needs
// (counts, slots) is updated here.
template <bool F32>
__device__ void commit(BlockShared<F32> &B, const ChainArrays &CA, int chain, int &st,
                       bool defer = false) {
  SysDev &S = B.S;
  ChainHdr &H = B.H;
  MoveCtx &mc = B.mc;
  const int accepted = mc.accepted && mc.kind != 0;  // a switch no-op keeps a stale `accepted`
  __syncthreads();  // every thread has read the decision before anyone moves on
  if (!accepted) return;
  const GuestType &G = S.g[mc.g];
  const int g = mc.g;
  if constexpr (!F32) {
    double2 *skg = CA.sk + ((size_t)chain * kMaxG + g) * CA.nkmax;
    const double2 *snew = CA.snew + (size_t)chain * CA.nkmax;
    const double2 *sold = CA.sold + (size_t)chain * CA.nkmax;
    int kb, ke;
    share_of(S.nk, B.ev.rank, B.ev.csize, kb, ke);
    for (int k = kb + threadIdx.x; k < ke; k += kThreads) {
      double2 v = skg[k], n = snew[k];
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
    }
  } else {
    // the evaluation wrote the updated S(k) to the other buffer
    if (threadIdx.x == 0) B.H.skb[g] ^= 1;
  }
  // molecule order and coordinates
  int *ord = CA.ord + ((size_t)chain * kMaxG + g) * CA.cap;
  int *freel = CA.freel + ((size_t)chain * kMaxG + g) * CA.cap;
  const bool res = F32 && CA.resident;
  if (res) {
    // shared-memory copy, molecule order: insertion appends, deletion shifts
    // the later molecules down (mc_moves.f:574-590), displacement overwrites
    const int n = H.nummols[g], ns = G.ns;
    if (threadIdx.x == 0) {
      int slot = mc.slot;
      if (mc.kind == 1) {
        slot = n < CA.cap ? n : -1;
        if (slot < 0) st |= kStCapacity;
      }
      B.flags[1] = slot;
    }
    __syncthreads();
    if (mc.kind == 2) {
      const int from = (mc.choice - 1) * ns, cnt = (n - mc.choice) * ns;
      for (int base = 0; base < cnt; base += kThreads) {
        const int j = base + threadIdx.x;
        float4 vh = make_float4(0.f, 0.f, 0.f, 0.f), vl = vh;
        if (j < cnt) {
          vh = B.grh[from + j + ns];
          vl = B.grl[from + j + ns];
        }
        __syncthreads();
        if (j < cnt) {
          B.grh[from + j] = vh;
          B.grl[from + j] = vl;
        }
        __syncthreads();
      }
    } else if (B.flags[1] >= 0 && threadIdx.x < 3 * ns) {
      const int s = threadIdx.x / 3, d = threadIdx.x % 3, i = B.flags[1];
      reinterpret_cast<float *>(&B.grh[i * ns + s])[d] = B.ev.phi[0][s][d];
      reinterpret_cast<float *>(&B.grl[i * ns + s])[d] = B.ev.plo[0][s][d];
      if (d == 0) {
        const float qh = (float)G.q[s];
        B.grh[i * ns + s].w = qh;
        B.grl[i * ns + s].w = (float)(G.q[s] - (double)qh);
      }
    }
  }
  if (!res && threadIdx.x == 0) {
    int slot = mc.slot;
    if (mc.kind == 1) {
      if (H.nfree[g] > 0) slot = freel[--H.nfree[g]];
      else if (H.nslots[g] < CA.cap) slot = H.nslots[g]++;
      else {
        st |= kStCapacity;
        slot = -1;
      }
      if (slot >= CA.cap || slot < -1) {  // a damaged free list
        st |= kStIndex;
        slot = -1;
      }
      if (slot >= 0 && B.ev.rank == 0) ord[H.nummols[g]] = slot;
    }
    B.flags[1] = slot;
  }
  __syncthreads();
  const int slot = B.flags[1];
  if (mc.kind == 2 && B.ev.rank == 0 && !res) {
    // remove entry choice-1 from the order list (mc_moves.f:574-590)
    int n = H.nummols[g];
    int c0 = mc.choice - 1;
    constexpr int kPer = 8;  // capacity <= 4096 = 8 * kThreads
    int vals[kPer];
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
      const int i = c0 + threadIdx.x + j * kThreads;
      if (i < n - 1) vals[j] = ord[i + 1];
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
      const int i = c0 + threadIdx.x + j * kThreads;
      if (i < n - 1) ord[i] = vals[j];
    }
    __syncthreads();
  }
  if (slot >= 0 && (mc.kind == 1 || mc.kind >= 3) && threadIdx.x < 3 * G.ns && B.ev.rank == 0 && !res) {
    int s = threadIdx.x / 3, d = threadIdx.x % 3;
    size_t b = gslot_base(CA, chain, g, slot) + s;
    if constexpr (F32) {  // the evaluated position is the hi/lo pair
      const float h = B.ev.phi[0][s][d], l = B.ev.plo[0][s][d];
      CA.gpos[b * 3 + d] = (double)h + (double)l;
      reinterpret_cast<float *>(CA.ghi + b)[d] = h;
      reinterpret_cast<float *>(CA.glo + b)[d] = l;
    } else {
      double v = mc.pos[0][s][d];
      CA.gpos[b * 3 + d] = v;
      float h = (float)v;
      reinterpret_cast<float *>(CA.ghi + b)[d] = h;
      reinterpret_cast<float *>(CA.glo + b)[d] = (float)(v - (double)h);
    }
    if (d == 0) {
      const float qh = (float)G.q[s];
      reinterpret_cast<float *>(CA.ghi + b)[3] = qh;
      reinterpret_cast<float *>(CA.glo + b)[3] = (float)(G.q[s] - (double)qh);
    }
  }
  if (threadIdx.x == 0 && slot >= 0) {
    const int mol = G.mol, n_old = H.nummols[g];
    if (defer) {
      auto &D = B.dfr;
      D.booked = 1;
      D.n_old = n_old;
      D.chgtmp = mc.chgtmp;
      D.surf_new = mc.surf_new;
      D.surf_old = mc.surf_old;
      for (int m = 0; m <= S.maxmls; ++m) D.delE[m] = mc.delE[m];
    } else {
      bookkeep<F32>(S, H, g, n_old, mc.kind, mc.delE, mc.chgtmp, mc.surf_new, mc.surf_old);
    }
    if (mc.kind == 1 || mc.kind == 2) {
      int sg = mc.kind == 1 ? 1 : -1;
      for (int s = 0; s < G.ns; ++s) {
        int ka = G.type[s];
        H.numtyp[ka] += sg;
        H.numtyp_mol[mol][ka] += sg;
        if (G.frz[s]) {
          H.numfrz[ka] += sg;
          H.numfrz_mol[mol][ka] += sg;
        }
      }
      H.nummols[g] += sg;
      if (mc.kind == 2 && !res) {
        if (B.ev.rank == 0) freel[H.nfree[g]] = slot;
        H.nfree[g]++;
      }
    }
  }
  __syncthreads();
  if (!res) cluster_commit_sync(B, st);  // resident guests: every CTA updated its own copy
}

// commit, called rather than inlined, for the seldom-run paths (as
// evaluate_rare).
template <bool F32>
__device__ __noinline__ void commit_rare(BlockShared<F32> &B, const ChainArrays &CA, int chain,
                                         int &st) {
  commit(B, CA, chain, st, false);
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

// Thread 0: acceptance counters (the next move's step-size adaptation reads
// them), then the production statistics, now or (defer) by run_deferred.
template <bool F32>
__device__ void stats_production(const SysDev &S, ChainHdr &H, int production, int accepted);

template <bool F32>
__device__ void stats(BlockShared<F32> &B, bool defer = false) {
  SysDev &S = B.S;
  ChainHdr &H = B.H;
  MoveCtx &mc = B.mc;
  int g = mc.g;
  H.last_accepted = mc.accepted;
  if (mc.accepted && mc.kind >= 1) {
    if (mc.kind == 1) H.accept_ins[g]++;
    else if (mc.kind == 2) H.accept_del[g]++;
    else if (mc.kind == 4) H.accept_tran[g]++;
    else if (mc.kind == 5) H.accept_rota[g]++;
    else if (mc.kind == 6) H.accept_jump[g]++;
    else H.accept_disp[g]++;
  }
  if (mc.kind >= 1) {
    H.attempts[mc.kind - 1]++;
    if (mc.accepted) H.accepts[mc.kind - 1]++;
  }
  H.moves++;
  if (defer) {
    B.dfr.production = H.production;
    B.dfr.pending = 1;
    return;
  }
  stats_production<F32>(S, H, H.production, mc.accepted);
}

// Production statistics of one move (gcmc.f:1047-1127).
template <bool F32>
__device__ void stats_production(const SysDev &S, ChainHdr &H, int production, int accepted) {
  if (!production) return;
  if (S.laccsample && !accepted) return;
  H.prodcount++;
  H.rollcount++;
  if (F32 && !S.laccsample) {
    H.pend++;
  } else {
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
  }
  if (--H.window_left == 0) {  // prodcount is a multiple of nwindsteps
    H.window_left = S.nwindsteps;
    flush_stats(S, H);
    double rc = double(H.rollcount);
    H.wsum += rc;
    for (int i = 0; i < S.ntpguest; ++i) {
      double aN = H.chainstats[i][0] / rc, E = H.chainstats[i][1] / rc,
             EN = H.chainstats[i][2] / rc, N2 = H.chainstats[i][3] / rc,
             E2 = H.chainstats[i][4] / rc, NF = H.chainstats[i][5] / rc;
      double w[8] = {aN, E, EN, N2, E2, NF, calc_qst(E, aN, N2, EN, S.temp),
                     calc_cv(E2, E, aN, N2, EN, S.temp)};
      for (int q = 0; q < 8; ++q) H.wacc[i][q] += rc * w[q];
      H.wsq[i] += rc * (aN * aN);
      for (int q = 0; q < 6; ++q) H.chainstats[i][q] = 0.0;
    }
    H.windows++;
    H.rollcount = 0;
  }
}

// Thread 32: the previous move's deferred FP64 work, in the order the
// reference does it (delE of the other molecule types, accept_move's
// updates, the production sums).  It reads the previous evaluation's block
// totals, which stay in ev.out until the next evaluation's reduction, and
// touches no field the proposal reads.
template <bool F32, int GN>
__device__ void run_deferred(BlockShared<F32> &B) {
  auto &D = B.dfr;
  if (!D.pending) return;
  if (D.other) other_mol_delE<F32, GN>(B, D.kind, D.g, D.npos, D.delE);
  if (D.booked)
    bookkeep<F32>(B.S, B.H, D.g, D.n_old, D.kind, D.delE, D.chgtmp, D.surf_new, D.surf_old);
  stats_production<F32>(B.S, B.H, D.production, D.accepted);
  D.pending = 0;
}

// ------------------------------------------------- speculative proposals
// Most trial moves of a dense framework end on the overlap test, change no
// state and consume a fixed number of generator draws (the Metropolis
// number is drawn only after the test passes, gcmc.f:1732).  So the next
// moves of a chain can be proposed ahead and their overlap tests run
// together: the proposals up to the first that passes (or that has no
// overlap test: a deletion, a switch that does nothing) are the chain's
// next moves exactly as the one-at-a-time loop would make them.  The ones
// before it are completed as overlap exits; the selections after it are
// undone (counters, step sizes, generator position).  FP32 chains of one
// guest type with cell lists and resident guests, no probability grids.

// The selection state select_move changes (one guest type).
template <bool F32>
__device__ __forceinline__ void save_selection(const BlockShared<F32> &B,
                                               typename BlockShared<F32>::SelState &s) {
  const ChainHdr &H = B.H;
  s.gcmccount = H.gcmccount;
  s.ins = H.ins_count[0];
  s.del = H.del_count[0];
  s.disp = H.disp_count[0];
  s.tran = H.tran_count[0];
  s.rota = H.rota_count[0];
  s.jump = H.jump_count[0];
  s.minchk_left = H.minchk_left;
  s.production = H.production;
  s.disp_mod = H.disp_mod[0];
  s.tran_mod = H.tran_mod[0];
  s.rota_mod = H.rota_mod[0];
  s.rhead = H.rhead;
  s.ravail = H.ravail;
  s.status = H.status;
  s.delrdisp = H.delrdisp[0];
  s.tran_delr = H.tran_delr[0];
  s.rotangle = H.rotangle;
  s.rota_rotangle = H.rota_rotangle;
  for (int i = 0; i < 2; ++i) {
    s.sh_disp[i] = H.sh_disp[0][i];
    s.sh_tran[i] = H.sh_tran[0][i];
    s.rho_rot[0][i] = H.rho_rot[0][i];
    s.rho_rot[1][i] = H.rho_rot[1][i];
  }
}

template <bool F32>
__device__ __forceinline__ void load_selection(BlockShared<F32> &B,
                                               const typename BlockShared<F32>::SelState &s) {
  ChainHdr &H = B.H;
  H.gcmccount = s.gcmccount;
  H.ins_count[0] = s.ins;
  H.del_count[0] = s.del;
  H.disp_count[0] = s.disp;
  H.tran_count[0] = s.tran;
  H.rota_count[0] = s.rota;
  H.jump_count[0] = s.jump;
  H.minchk_left = s.minchk_left;
  H.production = s.production;
  H.disp_mod[0] = s.disp_mod;
  H.tran_mod[0] = s.tran_mod;
  H.rota_mod[0] = s.rota_mod;
  H.rhead = s.rhead;
  H.ravail = s.ravail;
  H.status = s.status;
  H.delrdisp[0] = s.delrdisp;
  H.tran_delr[0] = s.tran_delr;
  H.rotangle = s.rotangle;
  H.rota_rotangle = s.rota_rotangle;
  for (int i = 0; i < 2; ++i) {
    H.sh_disp[0][i] = s.sh_disp[i];
    H.sh_tran[0][i] = s.sh_tran[i];
    H.rho_rot[0][i] = s.rho_rot[0][i];
    H.rho_rot[1][i] = s.rho_rot[1][i];
  }
}

// True when a chain can run speculative rounds (all threads agree).
template <bool F32>
__device__ __forceinline__ bool speculation_applies(const BlockShared<F32> &B, const ChainArrays &CA) {
  const SysDev &S = B.S;
  if (!F32 || CA.spec_max < 2 || !CA.resident || !S.use_cells || S.ntpguest != 1) return false;
  if (S.prob_nsub > 0 && CA.grid) return false;
  const float mincs = fminf(S.cszf[0], fminf(S.cszf[1], S.cszf[2]));
  return mincs >= sqrtf(S.overlap_sqf) + 0.01f;  // the 27 neighbour cells cover the test
}

// Overlap tests of the testable proposals of a round, all threads: every
// site against the 27 neighbour cells (padded slots) and every resident
// guest molecule, the arithmetic of overlap_check.  Sets spec[j].hit.
template <bool F32>
__device__ void overlap_batch(BlockShared<F32> &B, int n) {
  const SysDev &S = B.S;
  const int ns = S.g[0].ns, lp = S.cpad_log2;
  const int per = (ns * 27) << lp;
  for (int t = threadIdx.x; t < n * per; t += kThreads) {
    const int jp = t / per, r = t - jp * per;
    auto &P = B.spec[jp];
    if (!P.testable || *(volatile int *)&P.hit) continue;
    const int j = r & ((1 << lp) - 1);
    const int sc = r >> lp;
    const int s = sc / 27, c = sc - 27 * s;
    const int o3[3] = {c / 9 - 1, (c / 3) % 3 - 1, c % 3 - 1};
    int im[3], iw[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      int ic = (int)floorf(P.phi[0][s][d] * S.rcszf[d]) + o3[d];
      int k = 0;
      if (ic < 0) k = -1;
      else if (ic >= S.nc[d]) k = 1;
      if (ic - k * S.nc[d] < 0 || ic - k * S.nc[d] >= S.nc[d]) k = image_of(ic, S.nc[d]);
      im[d] = k;
      iw[d] = ic - k * S.nc[d];
    }
    const size_t a = ((size_t)((iw[0] * S.nc[1] + iw[1]) * S.nc[2] + iw[2]) << lp) + j;
    const float4 H4 = __ldg(S.cpad_hi + a), L4 = __ldg(S.cpad_lo + a);
    float ah[3] = {H4.x, H4.y, H4.z}, al[3] = {L4.x, L4.y, L4.z};
    float r2 = 0.f;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (im[d] != 0) {
        float h, e;
        two_sum_f(ah[d], float(im[d]) * S.boxh[d], h, e);
        ah[d] = h;
        al[d] = al[d] + (e + float(im[d]) * S.boxl[d]);
      }
      float dd = (P.phi[0][s][d] - ah[d]) + (P.plo[0][s][d] - al[d]);
      r2 = fmaf(dd, dd, r2);
    }
    if (r2 < S.overlap_sqf) P.hit = 1;
  }
  // resident guests, one (proposal, molecule) per item
  const GuestType &G = S.g[0];
  const int n2 = B.H.nummols[0];
  const float pre = sqrtf(S.overlap_sqf) + 2.0f * (float)G.rmax + 2.0f * (float)G.rmax + 0.01f;
  const float pre2 = pre * pre;
  for (int t = threadIdx.x; t < n * n2; t += kThreads) {
    const int jp = t / n2, i = t - jp * n2;
    auto &P = B.spec[jp];
    if (!P.testable || *(volatile int *)&P.hit) continue;
    if (P.kind != 1 && i == P.slot) continue;  // the moving molecule itself
    const float4 q0 = B.grh[i * ns];
    float dx = P.phi[0][0][0] - q0.x, dy = P.phi[0][0][1] - q0.y, dz = P.phi[0][0][2] - q0.z;
    dx -= S.boxh[0] * rint_image(dx * S.rboxf[0]);
    dy -= S.boxh[1] * rint_image(dy * S.rboxf[1]);
    dz -= S.boxh[2] * rint_image(dz * S.rboxf[2]);
    if (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) > pre2) continue;
    int hit = 0;
    for (int b = 0; b < ns; ++b) {
      const float4 qh = B.grh[i * ns + b], ql = B.grl[i * ns + b];
      for (int s = 0; s < ns; ++s) {
        float ex = mi_diff32(P.phi[0][s][0], P.plo[0][s][0], qh.x, ql.x, S.boxh[0], S.boxl[0], S.rboxf[0]);
        float ey = mi_diff32(P.phi[0][s][1], P.plo[0][s][1], qh.y, ql.y, S.boxh[1], S.boxl[1], S.rboxf[1]);
        float ez = mi_diff32(P.phi[0][s][2], P.plo[0][s][2], qh.z, ql.z, S.boxh[2], S.boxl[2], S.rboxf[2]);
        if (fmaf(ex, ex, fmaf(ey, ey, ez * ez)) < S.overlap_sqf) hit = 1;
      }
    }
    if (hit) P.hit = 1;
  }
}

// One speculative round of up to kwin proposals (all threads; ends with a
// barrier).  The overlap exits among them are completed here (counters,
// production statistics, log); the first proposal that is not one is left
// in mc / draws / ev as propose() leaves a move (spec_have = 1), with
// flags[6] set when its overlap test has passed.  Returns the exits.
template <bool F32, bool TRIC>
__device__ int spec_round(BlockShared<F32> &B, const ChainArrays &CA, int chain, int kwin,
                          LogRec *logs, int logcap, int rank) {
  SysDev &S = B.S;
  ChainHdr &H = B.H;
  MoveCtx &mc = B.mc;
  if (threadIdx.x < 32) {
    // draws for kwin proposals (at most 11 each) and the chosen one's
    // Metropolis number, within the ring
    const int need = 11 * kwin + 5;
    while (H.ravail < need) refill_draws(H);
    if (threadIdx.x == 0) {
      int n = 0;
      for (int j = 0; j < kwin; ++j) {
        mc.rande = -1.0;
        mc.estep = 0.0;
        mc.overlap = 0;
        mc.accepted = 0;
        mc.surf_new = mc.surf_old = 0;
        B.flags[5] = 0;
        select_move(B, CA, chain);
        if (mc.kind == 2 || (mc.kind >= 3 && mc.kind != 7)) {
          if (mc.choice < 1 || mc.choice > H.nummols[0]) {
            H.status |= kStBadChoice;
            mc.kind = 0;
          } else {
            mc.slot = mc.choice - 1;  // resident guests: molecule i in slot i
          }
        }
        auto &P = B.spec[j];
        P.kind = mc.kind;
        P.choice = mc.choice;
        P.slot = mc.slot;
        P.npos = mc.npos;
        P.flag2 = B.flags[2];
        P.flag5 = B.flags[5];
        P.production = H.production;
        for (int i = 0; i < 7; ++i) P.draws[i] = B.draws[i];
        for (int i = 0; i < 4; ++i) P.stepf[i] = B.stepf[i];
        P.testable = mc.kind == 1 || (mc.kind >= 3 && mc.kind <= 6);
        P.hit = 0;
        save_selection(B, P.sel);
        ++n;
        if (!P.testable) break;  // a deletion or a no-op: no test, it is this round's move
      }
      B.spec_n = n;
    }
  }
  __syncthreads();
  FMC_PHASE(B, 12);
  const int n = B.spec_n;
  {  // first-pass positions, warp j for proposal j
    const int w = threadIdx.x >> 5;
    if (w < n) {
      auto &P = B.spec[w];
      if (P.kind != 0)
        geometry_f32_core<F32, TRIC>(B, CA, chain, P.kind, 0, P.slot, P.draws, P.stepf, P.flag2, P.phi,
                                     P.plo);
    }
  }
  __syncthreads();
  FMC_PHASE(B, 13);
  overlap_batch(B, n);
  __syncthreads();
  FMC_PHASE(B, 14);
  if (threadIdx.x == 0) {
    int j = 0;
    const GuestType &G = S.g[0];
    while (j < n && B.spec[j].testable && B.spec[j].hit) {  // overlap exits
      const auto &P = B.spec[j];
      H.last_accepted = 0;
      H.attempts[P.kind - 1]++;
      H.moves++;
      H.overlap_exits++;
      if (logcap > 0 && H.log_n < logcap) {
        if (rank == 0) {
          LogRec &L = logs[(size_t)chain * logcap + H.log_n];
          L.move = P.kind;
          L.iguest = 1;
          L.choice = P.choice;
          L.overlap = 1;
          L.accepted = 0;
          L.estep = 0.0;
          L.rande = -1.0;
          for (int s = 0; s < 3 && s < G.ns; ++s)
            for (int d = 0; d < 3; ++d)
              L.newxyz[3 * s + d] = (double)P.phi[0][s][d] + (double)P.plo[0][s][d];
          L.nmols_after = H.nummols[0];
        }
        H.log_n++;
      }
      stats_production<F32>(S, H, P.production, 0);
      ++j;
    }
    B.spec_exits = j;
    B.spec_have = j < n;
    if (j < n) {  // the round's move: its selection state, the later ones undone
      const auto &P = B.spec[j];
      load_selection(B, P.sel);
      mc.kind = P.kind;
      mc.g = 0;
      mc.ns = G.ns;
      mc.choice = P.choice;
      mc.slot = P.slot;
      mc.npos = P.npos;
      mc.rande = -1.0;
      mc.estep = 0.0;
      mc.overlap = 0;
      mc.accepted = 0;
      mc.surf_new = mc.surf_old = 0;
      for (int i = 0; i < 7; ++i) B.draws[i] = P.draws[i];
      for (int i = 0; i < 4; ++i) B.stepf[i] = P.stepf[i];
      B.flags[2] = P.flag2;
      B.flags[5] = P.flag5;
      B.flags[3] = 1;  // FP32 first-pass geometry, refined after the test
      B.flags[4] = 1;  // delE of the other molecule types only if accepted
      B.flags[6] = P.testable;
    }
  }
  __syncthreads();
  if (B.spec_have && threadIdx.x < 32) {
    const auto &P = B.spec[B.spec_exits];
    const int lane = threadIdx.x, ns = S.g[0].ns;
    if (P.kind != 0 && lane < 3 * ns) {
      const int s = lane / 3, d = lane % 3;
      for (int p = 0; p < P.npos; ++p) {
        B.ev.phi[p][s][d] = P.phi[p][s][d];
        B.ev.plo[p][s][d] = P.plo[p][s][d];
      }
    }
    __syncwarp();
    if (P.kind != 0) site_constants_and_bounds(B);
  }
  __syncthreads();
  FMC_PHASE(B, 15);
  return B.spec_exits;
}

// Thread 0: the chain's counts, energies, charges, surface tallies and
// site-type counters, kept for a swap or switch that may be rejected, and
// put back.
template <bool F32>
__device__ void save_counts(BlockShared<F32> &B) {
  const ChainHdr &H = B.H;
  auto &W = B.swp;
  for (int g = 0; g < kMaxG; ++g) {
    W.nummols[g] = H.nummols[g];
    W.nslots[g] = H.nslots[g];
    W.nfree[g] = H.nfree[g];
    W.skb[g] = H.skb[g];
  }
  for (int m = 0; m <= kMaxM; ++m) {
    W.energy[m] = H.energy[m];
    W.chgsum_mol[m] = H.chgsum_mol[m];
    W.surfacemols[m] = H.surfacemols[m];
    for (int t = 0; t <= kMaxT; ++t) {
      W.numtyp_mol[m][t] = H.numtyp_mol[m][t];
      W.numfrz_mol[m][t] = H.numfrz_mol[m][t];
    }
  }
  for (int t = 0; t <= kMaxT; ++t) {
    W.numtyp[t] = H.numtyp[t];
    W.numfrz[t] = H.numfrz[t];
  }
}

template <bool F32>
__device__ void restore_counts(BlockShared<F32> &B) {
  ChainHdr &H = B.H;
  const auto &W = B.swp;
  for (int g = 0; g < kMaxG; ++g) {
    H.nummols[g] = W.nummols[g];
    H.nslots[g] = W.nslots[g];
    H.nfree[g] = W.nfree[g];
    H.skb[g] = W.skb[g];  // FP32: the buffers current before the move
  }
  for (int m = 0; m <= kMaxM; ++m) {
    H.energy[m] = W.energy[m];
    H.chgsum_mol[m] = W.chgsum_mol[m];
    H.surfacemols[m] = W.surfacemols[m];
    for (int t = 0; t <= kMaxT; ++t) {
      H.numtyp_mol[m][t] = W.numtyp_mol[m][t];
      H.numfrz_mol[m][t] = W.numfrz_mol[m][t];
    }
  }
  for (int t = 0; t <= kMaxT; ++t) {
    H.numtyp[t] = W.numtyp[t];
    H.numfrz[t] = W.numfrz[t];
  }
}

// All threads of rank 0's CTA: a deleted molecule's slot back into its
// type's order list at entry choice-1, the later entries shifted up (the
// deletion shifted them down, mc_moves.f:574-590); n is the count before
// the deletion.  Entry n-1, if in use, is overwritten.
__device__ inline void reinsert_order(const ChainArrays &CA, int chain, int g, int choice, int slot,
                               int n) {
  int *ord = CA.ord + ((size_t)chain * kMaxG + g) * CA.cap;
  const int c0 = choice - 1;
  constexpr int kPer = 8;  // capacity <= 4096 = 8 * kThreads
  int vals[kPer];
#pragma unroll
  for (int j = 0; j < kPer; ++j) {
    const int i = c0 + threadIdx.x + j * kThreads;
    if (i < n - 1) vals[j] = ord[i];
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kPer; ++j) {
    const int i = c0 + threadIdx.x + j * kThreads;
    if (i < n - 1) ord[i + 1] = vals[j];
  }
  if (threadIdx.x == 0) ord[c0] = slot;
  __syncthreads();
}

// This CTA's share of two guest types' S(k): the current buffers into the
// chain's save area (save) or the save area back into the buffers given
// by skb (restore).  FP32 entries are hi/lo float4, FP64 double2; both are
// 16 bytes, the save area is typed double2.
template <bool F32>
__device__ void sk_pair_copy(BlockShared<F32> &B, const ChainArrays &CA, int chain, int ga, int gb,
                             const int *skb, bool save) {
  const SysDev &S = B.S;
  int kb, ke;
  share_of(S.nk, B.ev.rank, B.ev.csize, kb, ke);
  const int gs[2] = {ga, gb};
  for (int m = 0; m < 2; ++m) {
    const size_t o = ((size_t)chain * kMaxG + gs[m]) * CA.nkmax;
    double2 *sv = CA.sksave + ((size_t)chain * 2 + m) * CA.nkmax;
    if constexpr (F32) {
      float4 *sk = (skb[gs[m]] ? CA.skdf2 : CA.skdf) + o;
      float4 *sv4 = reinterpret_cast<float4 *>(sv);
      for (int k = kb + threadIdx.x; k < ke; k += kThreads) {
        if (save) sv4[k] = sk[k];
        else sk[k] = sv4[k];
      }
    } else {
      double2 *sk = CA.sk + o;
      for (int k = kb + threadIdx.x; k < ke; k += kThreads) {
        if (save) sv[k] = sk[k];
        else sk[k] = sv[k];
      }
    }
  }
}

// mc_swap (gcmc.f:2269-2452) inside a device-resident chain, all threads:
// the chosen molecule of guest type g is deleted and the deletion committed
// (accept_move), a molecule of the partner type gj is built from its
// template at the deleted molecule's centre of mass, rotated about it by the
// drawn quaternion, inserted and committed, and the pair is decided by the
// reference's two tests (volume in cubic angstroms as written there; the
// second number is drawn only when the first test passes, neither when the
// insertion overlaps).  A rejection puts back what the reference's
// reject_move restores (mc_moves.f:646-669): coordinates, molecule order,
// S(k), counts, charges, surface tally and energies -- but not the system
// charge sumchg, which keeps the two commits as in the reference.  The
// reference also commits an overlapping insertion before undoing it; here
// it is not committed, which leaves the same state.
template <bool F32, int GN>
__device__ void swap_move(BlockShared<F32> &B, const ChainArrays &CA, int chain, int &st,
                          LogRec *logs, int logcap, int rank) {
  SysDev &S = B.S;
  ChainHdr &H = B.H;
  MoveCtx &mc = B.mc;
  auto &W = B.swp;
  const int gi = mc.g, gj = W.gj, choice = mc.choice, slot_i = mc.slot;
  const GuestType &Gi = S.g[gi], &Gj = S.g[gj];
  if (threadIdx.x == 0) {
    save_counts(B);
    // centre of mass of the chosen molecule (com, utility_pack.f:3565-3596)
    const double *src = CA.gpos + gslot_base(CA, chain, gi, slot_i) * 3;
    double w = 0.0, c[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < Gi.ns; ++k) {
      w += Gi.mass[k];
      for (int d = 0; d < 3; ++d) c[d] += src[3 * k + d] * Gi.mass[k];
    }
    for (int d = 0; d < 3; ++d) c[d] /= w;
    // the partner's template at c, rotated about c (rotation,
    // utility_pack.f:3480-3524): (t + c) - c as the reference forms it
    double q[4];
    draw_quaternion(B.draws, B.geo[7], q);
    for (int i = 0; i < Gj.ns; ++i) {
      double v[3];
      for (int d = 0; d < 3; ++d) v[d] = (Gj.tmpl[i][d] + c[d]) - c[d];
      for (int d = 0; d < 3; ++d) {
        double row[3];
        qrow(q, d, row);
        W.pos[i][d] = (row[0] * v[0] + row[1] * v[1] + row[2] * v[2]) + c[d];
      }
    }
    // the deletion first (forced commit: delE of every molecule type now)
    mc.kind = 2;
    mc.npos = 1;
    mc.ns = Gi.ns;
    B.flags[3] = F32 ? 1 : 0;
    B.flags[4] = 0;
    B.flags[6] = 0;
  }
  __syncthreads();
  // FP64: both types' S(k), this CTA's share, for a rejection (FP32: the
  // buffers the two evaluations do not write keep it)
  if constexpr (!F32) sk_pair_copy(B, CA, chain, gi, gj, H.skb, true);
  if (threadIdx.x < 32) {
    if constexpr (F32) geometry_f32<F32, kTricOk<F32, GN>>(B, CA, chain);
    else geometry_warp(B, CA, chain, kPropMC);
  }
  __syncthreads();
  evaluate_rare<F32, GN>(B, CA, chain, st);
  if (threadIdx.x == 0) {
    W.estepi = -mc.estep;
    mc.accepted = 1;
  }
  __syncthreads();
  commit_rare(B, CA, chain, st);
  // the partner molecule
  if (threadIdx.x == 0) {
    mc.kind = 1;
    mc.g = gj;
    mc.ns = Gj.ns;
    mc.npos = 1;
    mc.slot = -1;
    mc.choice = 0;
    mc.overlap = 0;
    mc.estep = 0.0;
    mc.surf_new = mc.surf_old = 0;
    for (int i = 0; i < Gj.ns; ++i)
      for (int d = 0; d < 3; ++d) mc.pos[0][i][d] = W.pos[i][d];
    B.flags[3] = 0;  // FP64 positions
    B.flags[4] = 0;
    B.flags[6] = 0;
  }
  __syncthreads();
  const int full_j = evaluate_rare<F32, GN>(B, CA, chain, st);
  if (threadIdx.x == 0) {
    W.estepj = mc.estep;
    W.overlap = mc.overlap;
    mc.accepted = mc.overlap ? 0 : 1;
  }
  __syncthreads();
  commit_rare(B, CA, chain, st);
  if (threadIdx.x == 0) {  // the reference's two tests (gcmc.f:2371-2411)
    int acc = 0;
    double r0 = -1.0;
    if (!W.overlap) {
      r0 = (double)draw_f(H);
      const int jn = H.nummols[gj], in = H.nummols[gi] + 1;
      const double testi = double(in) * kBoltz * S.temp / (S.volm * H.fuga[gi]) *
                           exp(-1.0 * S.beta * W.estepi);
      const double testj = S.volm * H.fuga[gj] / (double(jn) * kBoltz * S.temp) *
                           exp(-1.0 * S.beta * W.estepj);
      if (r0 < testi) acc = (double)draw_f(H) < testj;
    }
    W.accepted = acc;
    W.rande = r0;
  }
  __syncthreads();
  if (!W.accepted) {
    if (threadIdx.x == 0) restore_counts(B);  // FP32: skb back to the buffers left untouched
    if constexpr (!F32) sk_pair_copy(B, CA, chain, gi, gj, W.skb, false);
    // the deleted molecule back into the order list at its place
    if (rank == 0) reinsert_order(CA, chain, gi, choice, slot_i, W.nummols[gi]);
    __syncthreads();
    cluster_commit_sync(B, st);
  }
  if (threadIdx.x == 0) {
    const int acc = W.accepted;
    H.last_accepted = acc;
    H.attempts[6]++;
    if (acc) H.accepts[6]++;
    H.moves++;
    H.evals += 1 + (full_j ? 1 : 0);
    if (W.overlap) H.overlap_exits++;
    if (logcap > 0 && H.log_n < logcap) {
      if (rank == 0) {
        LogRec &L = logs[(size_t)chain * logcap + H.log_n];
        L.move = 7;
        L.iguest = gi + 1;
        L.choice = choice;
        L.overlap = W.overlap;
        L.accepted = acc;
        L.estep = W.estepi + W.estepj;
        L.rande = W.rande;
        for (int s = 0; s < 3 && s < Gj.ns; ++s)
          for (int d = 0; d < 3; ++d) L.newxyz[3 * s + d] = W.pos[s][d];
        L.nmols_after = H.nummols[gi];
      }
      H.log_n++;
    }
    mc.g = gi;  // the move's guest type, for what follows
    stats_production<F32>(S, H, H.production, acc);
  }
  __syncthreads();
}

// The acting mc_switch (gcmc.f:2096-2267) inside a device-resident chain,
// all threads: molecule ichoice of type gi and molecule jchoice of type gj
// exchange centres of mass, each keeping its orientation.  As the
// reference runs it: both deletions evaluated and committed (accept_move),
// the partner inserted at the first molecule's centre and committed, then
// the first molecule at the partner's centre, evaluated and committed.  An
// insertion that overlaps is committed too, as the reference does: it stops
// before its structure factor, so accept_move adds the one the partner's
// deletion left (FP64: the scratch s(k); FP32: the S(k) buffer that
// deletion did not write) and delE cleared, and the next insertion is
// evaluated against that state.  Decided as a displacement on estepi +
// estepj, with no number drawn when the sum is negative, and vetoed by any
// overlap.  A rejection puts back counts, energies, charges, surface
// tallies, both types' S(k), both molecules' coordinates and the order
// lists; the system charge keeps the four commits, which cancel.
template <bool F32, int GN>
__device__ void switch_move(BlockShared<F32> &B, const ChainArrays &CA, int chain, int &st,
                            LogRec *logs, int logcap, int rank) {
  SysDev &S = B.S;
  ChainHdr &H = B.H;
  MoveCtx &mc = B.mc;
  auto &W = B.swp;
  const int gi = mc.g, gj = W.gj, ichoice = mc.choice, jchoice = W.jchoice, slot_i = mc.slot;
  const GuestType &Gi = S.g[gi], &Gj = S.g[gj];
  if (threadIdx.x == 0) {
    save_counts(B);
    W.overlap = 0;
    W.slot_j = CA.ord[((size_t)chain * kMaxG + gj) * CA.cap + (jchoice - 1)];
    // both molecules' centres of mass (com, utility_pack.f:3565-3596), their
    // sites relative to them (gcmc.f:2140-2153) and their coordinates
    const int gs[2] = {gi, gj}, slots[2] = {slot_i, W.slot_j};
    for (int m = 0; m < 2; ++m) {
      const GuestType &G = S.g[gs[m]];
      const size_t b = gslot_base(CA, chain, gs[m], slots[m]);
      const double *src = CA.gpos + b * 3;
      double w = 0.0, c[3] = {0.0, 0.0, 0.0};
      for (int k = 0; k < G.ns; ++k) {
        w += G.mass[k];
        for (int d = 0; d < 3; ++d) c[d] += src[3 * k + d] * G.mass[k];
      }
      for (int d = 0; d < 3; ++d) W.cen[m][d] = c[d] / w;
      for (int k = 0; k < G.ns; ++k) {
        for (int d = 0; d < 3; ++d) {
          W.opos[m][k][d] = src[3 * k + d];
          W.rel[m][k][d] = src[3 * k + d] - W.cen[m][d];
        }
        W.ohi[m][k] = CA.ghi[b + k];
        W.olo[m][k] = CA.glo[b + k];
      }
    }
    mc.kind = 2;  // the first deletion (choice, slot as proposed)
    mc.npos = 1;
    mc.ns = Gi.ns;
    B.flags[3] = F32 ? 1 : 0;
    B.flags[4] = 0;  // delE of every molecule type now: the commit is forced
    B.flags[6] = 0;
  }
  __syncthreads();
  sk_pair_copy(B, CA, chain, gi, gj, H.skb, true);  // this CTA's share, for a rejection
  int nfull = 0;
  // step: evaluate the move in mc (positions from the geometry for a
  // deletion, given in mc.pos for an insertion) and commit it, forced
  auto half = [&](double &acc_estep, bool del) {
    if (del && threadIdx.x < 32) {
      if constexpr (F32) geometry_f32<F32, kTricOk<F32, GN>>(B, CA, chain);
      else geometry_warp(B, CA, chain, kPropMC);
    }
    __syncthreads();
    nfull += evaluate_rare<F32, GN>(B, CA, chain, st);
    if (threadIdx.x == 0) {
      if (del) {
        acc_estep = -mc.estep;
      } else if (mc.overlap) {
        W.overlap = 1;  // insertion cleared delE before its overlap exit; estep stays 0
        for (int m = 0; m <= kMaxM; ++m) mc.delE[m] = 0.0;
      } else {
        acc_estep += mc.estep;
      }
      mc.accepted = 1;
    }
    __syncthreads();
    commit_rare(B, CA, chain, st);
  };
  half(W.estepi, true);
  if (threadIdx.x == 0) {  // the partner's deletion
    mc.kind = 2;
    mc.g = gj;
    mc.ns = Gj.ns;
    mc.npos = 1;
    mc.choice = jchoice;
    mc.slot = W.slot_j;
    mc.overlap = 0;
    mc.estep = 0.0;
    mc.accepted = 0;
    mc.surf_new = mc.surf_old = 0;
    B.flags[3] = F32 ? 1 : 0;
  }
  half(W.estepj, true);
  // the partner at the first molecule's centre, then the first molecule at
  // the partner's (gcmc.f:2185-2214)
  for (int m = 1; m >= 0; --m) {
    if (threadIdx.x == 0) {
      const GuestType &G = m ? Gj : Gi;
      mc.kind = 1;
      mc.g = m ? gj : gi;
      mc.ns = G.ns;
      mc.npos = 1;
      mc.slot = -1;
      mc.choice = 0;
      mc.overlap = 0;
      mc.estep = 0.0;
      mc.accepted = 0;
      mc.surf_new = mc.surf_old = 0;
      for (int k = 0; k < G.ns; ++k)
        for (int d = 0; d < 3; ++d) mc.pos[0][k][d] = W.rel[m][k][d] + W.cen[1 - m][d];
      B.flags[3] = 0;  // FP64 positions
    }
    half(m ? W.estepj : W.estepi, false);
  }
  if (threadIdx.x == 0) {  // gcmc.f:2218-2229
    const double e = W.estepi + W.estepj;
    int acc = 1;
    double r0 = -1.0;
    if (!(e < 0.0)) {
      r0 = (double)draw_f(H);
      double test;
      if (-S.beta * e > 700.0) test = exp(700.0);
      else if (S.beta * e > 700.0) test = exp(-700.0);
      else test = exp(-1.0 * S.beta * e);
      acc = r0 < test;
    }
    if (W.overlap) acc = 0;
    W.accepted = acc;
    W.rande = r0;
  }
  __syncthreads();
  if (!W.accepted) {
    if (threadIdx.x == 0) restore_counts(B);
    sk_pair_copy(B, CA, chain, gi, gj, W.skb, false);
    if (rank == 0) {
      // order lists: each molecule back at its entry (its re-insertion took
      // the slot its deletion freed and sits at the end), and its coordinates
      reinsert_order(CA, chain, gi, ichoice, slot_i, W.nummols[gi]);
      reinsert_order(CA, chain, gj, jchoice, W.slot_j, W.nummols[gj]);
      const int t = threadIdx.x;
      if (t < 2 * kMaxS) {
        const int m = t / kMaxS, k = t % kMaxS;
        const GuestType &G = m ? Gj : Gi;
        if (k < G.ns) {
          const size_t b = gslot_base(CA, chain, m ? gj : gi, m ? W.slot_j : slot_i) + k;
          for (int d = 0; d < 3; ++d) CA.gpos[b * 3 + d] = W.opos[m][k][d];
          CA.ghi[b] = W.ohi[m][k];
          CA.glo[b] = W.olo[m][k];
        }
      }
    }
    __syncthreads();
    cluster_commit_sync(B, st);
  }
  if (threadIdx.x == 0) {
    const int acc = W.accepted;
    H.last_accepted = acc;
    H.attempts[7]++;
    if (acc) H.accepts[7]++;
    H.moves++;
    H.evals += nfull;
    if (W.overlap) H.overlap_exits++;
    if (logcap > 0 && H.log_n < logcap) {
      if (rank == 0) {
        LogRec &L = logs[(size_t)chain * logcap + H.log_n];
        L.move = 8;
        L.iguest = gi + 1;
        L.choice = ichoice;
        L.overlap = W.overlap;
        L.accepted = acc;
        L.estep = W.estepi + W.estepj;
        L.rande = W.rande;
        for (int k = 0; k < 3 && k < Gi.ns; ++k)
          for (int d = 0; d < 3; ++d) L.newxyz[3 * k + d] = W.rel[0][k][d] + W.cen[1][d];
        L.nmols_after = H.nummols[gi];
      }
      H.log_n++;
    }
    mc.g = gi;  // the move's guest type, for what follows
    stats_production<F32>(S, H, H.production, acc);
  }
  __syncthreads();
}

// equitable_bin (utility_pack.f:2407-2519) into one subgrid with atomics:
// val spread over the 2x2x2 voxels around a fractional point, including the
// reference's wraps (a b-direction offset of 1 at the upper edge).
__device__ inline void equitable_bin_dev(double *g, const int *ng, double fa, double fb,
                                         double fc, double val) {
  const int na = ng[0], nb = ng[1], nc = ng[2];
  int alidx, aridx, blidx, bridx, clidx, cridx;
  double al, ar, bl, br, cl, cr;
  const double gpta = na * fa;
  const int aidx = (int)ceil(gpta);
  const double apart = gpta - floor(gpta);
  if (apart > 0.5) {
    if (aidx >= na) {
      alidx = (na - 1) * nb * nc;
      aridx = 0;
    } else {
      alidx = (aidx - 1) * nb * nc;
      aridx = aidx * nb * nc;
    }
    al = 1.5 - apart;
    ar = apart - 0.5;
  } else {
    if (aidx <= 1) {
      alidx = (na - 1) * nb * nc;
      aridx = 0;
    } else {
      alidx = (aidx - 2) * nb * nc;
      aridx = (aidx - 1) * nb * nc;
    }
    al = 0.5 - apart;
    ar = 0.5 + apart;
  }
  const double gptb = nb * fb;
  const int bidx = (int)ceil(gptb);
  const double bpart = gptb - floor(gptb);
  if (bpart > 0.5) {
    if (bidx >= nb) {
      blidx = (nb - 1) * nc;
      bridx = 1;
    } else {
      blidx = (bidx - 1) * nc;
      bridx = bidx * nc;
    }
    bl = 1.5 - bpart;
    br = bpart - 0.5;
  } else {
    if (bidx <= 1) {
      blidx = (nb - 1) * nc;
      bridx = 0;
    } else {
      blidx = (bidx - 2) * nc;
      bridx = (bidx - 1) * nc;
    }
    bl = 0.5 - bpart;
    br = 0.5 + bpart;
  }
  const double gptc = nc * fc;
  const int cidx = (int)ceil(gptc);
  const double cpart = gptc - floor(gptc);
  if (cpart > 0.5) {
    if (cidx >= nc) {
      clidx = nc;
      cridx = 1;
    } else {
      clidx = cidx;
      cridx = cidx + 1;
    }
    cl = 1.5 - cpart;
    cr = cpart - 0.5;
  } else {
    if (cidx <= 1) {
      clidx = nc;
      cridx = 1;
    } else {
      clidx = cidx - 1;
      cridx = cidx;
    }
    cl = 0.5 - cpart;
    cr = 0.5 + cpart;
  }
  g -= 1;  // bins are 1-based
  atomicAdd(g + alidx + blidx + clidx, (al * bl * cl) * val);
  atomicAdd(g + aridx + blidx + clidx, (ar * bl * cl) * val);
  atomicAdd(g + alidx + bridx + clidx, (al * br * cl) * val);
  atomicAdd(g + alidx + blidx + cridx, (al * bl * cr) * val);
  atomicAdd(g + aridx + bridx + clidx, (ar * br * cl) * val);
  atomicAdd(g + aridx + blidx + cridx, (ar * bl * cr) * val);
  atomicAdd(g + alidx + bridx + cridx, (al * br * cr) * val);
  atomicAdd(g + aridx + bridx + cridx, (ar * br * cr) * val);
}

// storeenprob (utility_pack.f:550-618) as the main loop calls it after an
// accepted production move (gcmc.f:1131-1134): with the main program's
// randchoice and guest_toten, which no move routine sets (theirs are their
// own variables), so molecule 0 -- newx as the move left it -- and energy 0.
// The centre of mass of the move's last positions (the guest type's site
// count and masses), folded into the unit cell, adds 1 to the guest type's
// count grid; the energy grid gains 0 and is left alone.  Thread 0 of rank
// 0.  newx is position 0 of the last evaluation: the inserted, deleted or
// moved molecule, a swap's partner over the deleted molecule's later sites,
// a switch's first molecule at its new centre, and for a switch that did
// nothing the previous move's.  widom_grid (gcmc.f:2529-2532) calls it with
// a test insertion's estep: `energy` adds that to the energy grid too.
template <bool F32>
__device__ void store_enprob(BlockShared<F32> &B, const ChainArrays &CA, int chain, int g,
                             const double *energy = nullptr) {
  const SysDev &S = B.S;
  if (threadIdx.x != 0 || B.ev.rank != 0 || S.prob_eng_sub[g] < 0) return;
  const GuestType &G = S.g[g];
  double c[3] = {0.0, 0.0, 0.0}, w = 0.0;
  for (int k = 0; k < G.ns; ++k) {
    const double m = G.mass[k];
    w += m;
    for (int d = 0; d < 3; ++d) {
      const double x = F32 ? (double)B.ev.phi[0][k][d] + (double)B.ev.plo[0][k][d] : B.mc.pos[0][k][d];
      c[d] += x * m;
    }
  }
  for (int d = 0; d < 3; ++d) c[d] /= w;
  const double *r = S.rucell;  // frac2
  double fx = c[0] * r[0] + c[1] * r[3] + c[2] * r[6];
  double fy = c[0] * r[1] + c[1] * r[4] + c[2] * r[7];
  double fz = c[0] * r[2] + c[1] * r[5] + c[2] * r[8];
  fx -= floor(fx);
  fy -= floor(fy);
  fz -= floor(fz);
  double *grid = CA.grid + (size_t)chain * CA.grid_stride;
  if (energy)
    equitable_bin_dev(grid + (size_t)S.prob_eng_sub[g] * S.prob_gridsize, S.ngrid, fx, fy, fz,
                      *energy);
  equitable_bin_dev(grid + (size_t)(S.prob_eng_sub[g] + 1) * S.prob_gridsize, S.ngrid, fx, fy, fz,
                    1.0);
}

// storeprob (utility_pack.f:621-687), all threads after a production move:
// every molecule's centre of mass or listed sites, folded into the unit
// cell, binned with weight 1.  One work item per (molecule, item); the CTAs
// of a cluster take shares of the molecules.  FP64, as the reference (the
// bin choice depends on the last bits of the fractional position).
template <bool F32>
__device__ void store_prob(BlockShared<F32> &B, const ChainArrays &CA, int chain) {
  const SysDev &S = B.S;
  double *grid = CA.grid + (size_t)chain * CA.grid_stride;
  for (int g = 0; g < S.ntpguest; ++g) {
    const int nit = S.prob_nitem[g];
    if (nit == 0) continue;
    const GuestType &G = S.g[g];
    const int n = B.H.nummols[g], ns = G.ns;
    int i0, i1;
    share_of(n, B.ev.rank, B.ev.csize, i0, i1);
    const int *ord = CA.ord + ((size_t)chain * kMaxG + g) * CA.cap;
    for (int t = threadIdx.x; t < (i1 - i0) * nit; t += kThreads) {
      const int i = i0 + t / nit, it = S.prob_item0[g] + t % nit;
      const int site = S.prob_site[it];
      auto pos = [&](int sidx, int d) -> double {
        if constexpr (F32) {
          if (CA.resident) {
            const float4 h = B.grh[i * ns + sidx], l = B.grl[i * ns + sidx];
            return d == 0 ? (double)h.x + (double)l.x
                          : (d == 1 ? (double)h.y + (double)l.y : (double)h.z + (double)l.z);
          }
        }
        return CA.gpos[(gslot_base(CA, chain, g, ord[i]) + sidx) * 3 + d];
      };
      double px = 0.0, py = 0.0, pz = 0.0;
      if (site == 0) {  // com (utility_pack.f:3565-3598)
        double w = 0.0;
        for (int k = 0; k < ns; ++k) {
          const double m = G.mass[k];
          w += m;
          px += pos(k, 0) * m;
          py += pos(k, 1) * m;
          pz += pos(k, 2) * m;
        }
        px /= w;
        py /= w;
        pz /= w;
      } else {
        px = pos(site - 1, 0);
        py = pos(site - 1, 1);
        pz = pos(site - 1, 2);
      }
      const double *r = S.rucell;  // frac2 / frac: modulo 1 in the unit cell
      double fx = px * r[0] + py * r[3] + pz * r[6];
      double fy = px * r[1] + py * r[4] + pz * r[7];
      double fz = px * r[2] + py * r[5] + pz * r[8];
      fx -= floor(fx);
      fy -= floor(fy);
      fz -= floor(fz);
      equitable_bin_dev(grid + (size_t)S.prob_sub[it] * S.prob_gridsize, S.ngrid, fx, fy, fz, 1.0);
    }
  }
}

}  // namespace fmcdev

// chain_kernel.cuh -- the persistent chain kernel and the host wrappers each
// of its instantiations exports.  A chain runs on a cluster of `csize` CTAs
// (1 .. kMaxCluster): every CTA runs the same control flow on the same
// replicated state (generator, proposal, decision), takes its share of the
// framework atoms, guests and k-vectors, and the shares' totals are
// exchanged through distributed shared memory.  Rank 0 alone writes the
// chain's guest arrays, log and state record.  Every instantiation lives in
// its own translation unit (chain_*.cu) so they compile in parallel.
#pragma once

#include <cuda_runtime.h>

#include "engine.cuh"

namespace fmc {
using namespace fmcdev;

// Modes of the chain kernel.
constexpr int kModeMoves = 0;   // nmoves main-loop iterations
constexpr int kModeCreate = 1;  // "create molecules" pre-loading
constexpr int kModeEval = 2;    // evaluate the move in gctx (per-move ABI)
constexpr int kModeCommit = 3;  // decide with gctx.rande and commit
constexpr int kModeWidom = 4;   // test insertions of a WidomJob (no state change)
constexpr int kModeLoad = 5;    // insert a WidomJob's positions into chain wj.chain (restart)
// Widom screen: margin (A^2) on the overlap distance squared, far above the
// error of a float trial geometry (~1e-5 A in a 100 A cell); trials per
// warp between the block's barriers
constexpr float kScreenMargin = 1e-3f;

// Coordinate d of site s of trial t of a Widom job (FP64): the caller's
// position, or a grid point (1-based fractions) and a random orientation
// (random_rot with angle 2 pi, rotation about the origin).
__device__ __forceinline__ double widom_site(const SysDev &S, const GuestType &G, const WidomJob &wj,
                                             int t, int s, int d) {
  if (wj.xyz_in) return wj.xyz_in[((size_t)t * G.ns + s) * 3 + d];
  const int gi = t / wj.nstep;
  const int i = gi / (wj.ng[1] * wj.ng[2]) + 1, j = (gi / wj.ng[2]) % wj.ng[1] + 1, k = gi % wj.ng[2] + 1;
  const double f[3] = {double(i) / wj.ng[0], double(j) / wj.ng[1], double(k) / wj.ng[2]};
  float dr[7];
  for (int q = 3; q < 7; ++q) dr[q] = hash_uniform(wj.seed, 4ull * (unsigned long long)t + (q - 3));
  double qt[4], row[3];
  draw_quaternion(dr, 2.0 * kPi, qt);
  qrow(qt, d, row);
  const double *tp = G.tmpl[s];
  return row[0] * tp[0] + row[1] * tp[1] + row[2] * tp[2] + S.cell[d] * f[0] + S.cell[3 + d] * f[1] +
         S.cell[6 + d] * f[2];
}

// Warp 0: trial t of a Widom job as an external insertion (FP64 positions).
template <bool F32>
__device__ void widom_propose(BlockShared<F32> &B, const WidomJob &wj, int t) {
  const int lane = threadIdx.x & 31;
  MoveCtx &mc = B.mc;
  const SysDev &S = B.S;
  const GuestType &G = S.g[wj.iguest];
  const int ns = G.ns;
  if (lane == 0) {
    mc.kind = 1;
    mc.g = wj.iguest;
    mc.ns = ns;
    mc.npos = 1;
    mc.slot = -1;
    mc.choice = 0;
    mc.overlap = 0;
    mc.accepted = 0;
    mc.rande = -1.0;
    mc.estep = 0.0;
    mc.surf_new = mc.surf_old = 0;
    B.flags[3] = 0;  // FP64 positions: the evaluation converts them
    B.flags[4] = 1;  // no delE of other molecule types
    B.flags[6] = 0;
  }
  if (lane < 3 * ns) {
    const int s = lane / 3, d = lane % 3;
    const double v = widom_site(S, G, wj, t, s, d);
    mc.pos[0][s][d] = v;
    if (wj.xyz_out) wj.xyz_out[((size_t)t * ns + s) * 3 + d] = v;
  }
}

// Trial of warp w in round k of chunk c of this block: blocks take every
// gridDim-th group of kWarps trials, so the trials that need the full
// evaluation spread over the blocks as the grid points do.
__device__ __forceinline__ long long widom_trial(int c, int k, int w) {
  return ((long long)(c * kScreenPer + k) * gridDim.x + blockIdx.x) * kWarps + w;
}

// Widom jobs on the FP32 path: warp w screens its trials of chunk c (one
// per round k < kScreenPer) against the framework (27 neighbour cells) in
// float and records each either as an overlap or in wsc.list[k][w] for the
// full evaluation.  Several trials per warp between the block's barriers,
// so a warp whose trial needs the whole scan does not hold the others up.
// Out of line, so the screen's registers stay out of the move loop's
// allocation.
template <bool F32>
__device__ __noinline__ void widom_screen(BlockShared<F32> &B, const WidomJob &wj, int chunk) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const GuestType &G = B.S.g[wj.iguest];
  const int ns = G.ns, lp = B.S.cpad_log2;
  for (int kk = 0; kk < kScreenPer; ++kk) {
    const long long tl = widom_trial(chunk, kk, warp);
    if (lane == 0) B.wsc.list[kk][warp] = -1;
    if (tl >= wj.ntrial) continue;
    const int t = (int)tl;
    bool sane = true;
    if (lane < 3 * ns) {
      const int s = lane / 3, d = lane % 3;
      float v;
      if (wj.xyz_in) {
        v = (float)wj.xyz_in[((size_t)t * ns + s) * 3 + d];
      } else {
        const int gi = t / wj.nstep;
        const int i = gi / (wj.ng[1] * wj.ng[2]) + 1, j = (gi / wj.ng[2]) % wj.ng[1] + 1,
                  k = gi % wj.ng[2] + 1;
        const float f[3] = {(float)i / (float)wj.ng[0], (float)j / (float)wj.ng[1],
                            (float)k / (float)wj.ng[2]};
        float dr[7], q[4], row[3];
        for (int r = 3; r < 7; ++r)
          dr[r] = hash_uniform(wj.seed, 4ull * (unsigned long long)t + (r - 3));
        quat_f32(dr, 1.0f, q);  // random_rot with angle 2 pi
        qrow(q, d, row);
        const float *tp = B.wsc.tmpl[s], *cl = B.wsc.cell;
        v = row[0] * tp[0] + row[1] * tp[1] + row[2] * tp[2] + cl[d] * f[0] + cl[3 + d] * f[1] +
            cl[6 + d] * f[2];
      }
      B.wsc.pos[warp][s][d] = v;
      sane = fabsf(v) < 1.0e6f;  // NaN fails too
    }
    sane = __all_sync(0xffffffffu, sane);
    __syncwarp();
    bool hit = false;
    if (sane) {
      const float lim = B.S.overlap_sqf - kScreenMargin, zero[3] = {0.f, 0.f, 0.f};
      const int nitem = (ns * 27) << lp;
      // two slots per lane in flight, then stop at the first round that
      // found one (an overlapping trial usually does within its first
      // site's cells)
      for (int base = 0; base < nitem; base += 64) {
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int it = base + 32 * u + lane;
          if (it < nitem) {
            const int j = it & ((1 << lp) - 1), sc = it >> lp;
            const int s = sc / 27, c = sc - 27 * s;
            if (overlap_r2_27(B.S, B.wsc.pos[warp][s], zero, c, j) < lim) hit = true;
          }
        }
        if (__any_sync(0xffffffffu, hit)) break;
      }
    }
    hit = __any_sync(0xffffffffu, hit);
    if (lane == 0) {
      if (hit) {
        if (wj.estep_out) wj.estep_out[t] = 0.0;
        if (wj.overlap_out) wj.overlap_out[t] = 1;
        atomicAdd(&B.wsc.nscreened, 1);
      } else {
        B.wsc.list[kk][warp] = t;
      }
    }
    // the trial's positions as the full evaluation forms them
    if (hit && wj.xyz_out && lane < 3 * ns) {
      const int s = lane / 3, d = lane % 3;
      wj.xyz_out[((size_t)t * ns + s) * 3 + d] = widom_site(B.S, G, wj, t, s, d);
    }
    __syncwarp();  // the next trial's positions go where this one's were read
  }
}

template <class T>
__device__ void block_copy(T *dst, const T *src) {
  static_assert(sizeof(T) % 4 == 0, "copy granularity");
  const int *s = reinterpret_cast<const int *>(src);
  int *d = reinterpret_cast<int *>(dst);
  for (int i = threadIdx.x; i < (int)(sizeof(T) / 4); i += kThreads) d[i] = s[i];
}

template <bool F32, int GN>
__global__ void __launch_bounds__(kThreads, 1)
    chain_kernel(const SysDev *__restrict__ systems, ChainHdr *hdrs, ChainArrays CA,
                 MoveCtx *gctx, LogRec *logs, int logcap, int nmoves, int mode,
                 const double *__restrict__ ctl_fuga, const int *__restrict__ chain_ids,
                 int csize, WidomJob wj) {
  extern __shared__ __align__(16) unsigned char dyn[];
  BlockShared<F32> &B = *reinterpret_cast<BlockShared<F32> *>(dyn);
  const unsigned long long t_start = global_ns();
  const int rank = csize > 1 ? (int)cluster_rank() : 0;
  const int chain = (mode == kModeWidom || mode == kModeLoad)
                        ? wj.chain
                        : (chain_ids ? chain_ids[blockIdx.x / csize] : (int)blockIdx.x / csize);
  block_copy(&B.H, hdrs + chain);
  __syncthreads();
  block_copy(&B.S, systems + B.H.system);
  if (threadIdx.x == 0) {
    B.flags[0] = 0;
    if (ctl_fuga && mode == kModeMoves) B.H.fuga[0] = ctl_fuga[chain];  // host control block
    if constexpr (F32) {  // log of energy_eval's prefactor, for the FP32 decisions
      for (int g = 0; g < B.S.ntpguest; ++g) {
        const double x = B.S.statvolm * B.H.fuga[g] / (kBoltz * B.S.temp);
        B.H.lnpf[g] = x > 0.0 ? (float)log(x) : -INFINITY;
      }
    }
    B.ev.rank = rank;
    B.ev.csize = csize;
    B.ev.tabpos = mode == kModeWidom ? 1 : 2;
    B.xseq = B.cseq = 0u;
    B.cflag = 0u;
  }
  if (threadIdx.x < kMaxCluster) B.xflag[threadIdx.x] = 0u;
  if (threadIdx.x == 0) {
    B.si_g = -1;
    B.dfr.pending = 0;
  }
  if constexpr (F32) {
    for (int i = threadIdx.x; i < kTrigN; i += kThreads) B.trig[i] = CA.trig[i];
  }
  __syncthreads();  // the system record and header are complete
  if (F32 && CA.resident) {  // guests into shared memory, molecule order
    const int n = B.H.nummols[0], ns = B.S.g[0].ns;
    const int *ord = CA.ord + (size_t)chain * kMaxG * CA.cap;
    const float4 *gh = CA.ghi + (size_t)chain * kMaxG * CA.cap * kMaxS;
    const float4 *gl = CA.glo + (size_t)chain * kMaxG * CA.cap * kMaxS;
    for (int idx = threadIdx.x; idx < n * ns; idx += kThreads) {
      const int i = idx / ns, sidx = idx - i * ns;
      const size_t o = (size_t)ord[i] * kMaxS + sidx;
      B.grh[idx] = gh[o];
      B.grl[idx] = gl[o];
    }
  }
  __syncthreads();
  if (csize > 1) cluster_barrier();  // every CTA's flags are cleared before anyone posts
  int st = 0;
#ifdef FMC_PHASE_TIMERS
  if (threadIdx.x == 0) B.tmark = clock64();
#endif
  if (mode == kModeMoves) {
    // speculative rounds of up to kspec proposals where they apply; kspec
    // doubles after a round of exits only and halves after a round whose
    // first proposal passed (every thread computes the same value)
    // (one guest type only: compiled into the single-type kernel alone)
    const bool spec = GN == 1 && speculation_applies(B, CA);
    const int kcap = min(CA.spec_max, kMaxSpec);
    int kspec = 2;
    for (int it = 0; it < nmoves; ++it) {
      // the previous move's FP64 bookkeeping overlaps this proposal
      if (threadIdx.x == 32) run_deferred<F32, GN>(B);
      if (spec) {
        const int kwin = min(kspec, nmoves - it);
        int exits = 0;
        if constexpr (GN == 1)
          exits = spec_round<F32, kTricOk<F32, GN>>(B, CA, chain, kwin, logs, logcap, rank);
        it += exits;
        if (!B.spec_have) kspec = min(2 * kspec, kcap);
        else if (exits == 0) kspec = max(1, kspec / 2);
        if (!B.spec_have) {
          --it;  // the loop's increment counts no further move
          continue;
        }
      } else {
        propose<F32, kTricOk<F32, GN>>(B, CA, chain, kPropMC, 0);
      }
      FMC_PHASE(B, 0);
      if (B.mc.kind >= 7) {  // mc_swap / the acting mc_switch: evaluations, decision, commits or rollback, statistics
        // (two or more guest types: not compiled into the single-type kernel,
        // whose systems cannot draw them)
        if constexpr (GN > 1) {
          if (B.mc.kind == 7) swap_move<F32, GN>(B, CA, chain, st, logs, logcap, rank);
          else switch_move<F32, GN>(B, CA, chain, st, logs, logcap, rank);
        } else {
          st |= kStBadChoice;
        }
        if (B.S.prob_nsub > 0 && CA.grid && B.H.production) {
          store_prob(B, CA, chain);
          if (B.swp.accepted) store_enprob(B, CA, chain, B.mc.g);
        }
        __syncthreads();
        continue;
      }
      int full = 0;
      if (B.mc.kind != 0) full = evaluate_any<F32, GN>(B, CA, chain, st);
      if (threadIdx.x == 0) {
        decide(B, true);
        auto &D = B.dfr;
        D.kind = B.mc.kind;
        D.g = B.mc.g;
        D.npos = B.mc.npos;
        D.accepted = B.mc.accepted;
        D.other = B.mc.accepted && B.mc.kind != 0 && B.flags[4];  // delE of the other molecule types
        D.booked = 0;
        if (full) B.H.evals += B.mc.npos;
        else if (B.mc.overlap) B.H.overlap_exits++;
        if (logcap > 0 && B.H.log_n < logcap && rank == 0) {
          LogRec &L = logs[(size_t)chain * logcap + B.H.log_n];
          L.move = B.mc.kind;
          L.iguest = B.mc.g + 1;
          L.choice = B.mc.choice;
          L.overlap = B.mc.overlap;
          L.accepted = B.mc.accepted;
          L.estep = B.mc.estep;
          L.rande = B.mc.rande;
          for (int s = 0; s < 3 && s < B.mc.ns; ++s)
            for (int d = 0; d < 3; ++d)
              L.newxyz[3 * s + d] = F32 ? (double)B.ev.phi[0][s][d] + (double)B.ev.plo[0][s][d]
                                        : B.mc.pos[0][s][d];
        }
      }
      __syncthreads();
      FMC_PHASE(B, 9);
      commit(B, CA, chain, st, true);
      FMC_PHASE_SYNC(B, 10);
      if (threadIdx.x == 0) {
        stats(B, true);
        if (logcap > 0 && B.H.log_n < logcap) {
          if (rank == 0) logs[(size_t)chain * logcap + B.H.log_n].nmols_after = B.H.nummols[B.mc.g];
          B.H.log_n++;
        }
      }
      __syncthreads();
      // probability grids after every production move (gcmc.f:1129-1130)
      if (B.S.prob_nsub > 0 && CA.grid && B.dfr.production) {
        store_prob(B, CA, chain);
        if (B.mc.accepted) store_enprob(B, CA, chain, B.mc.g);
      }
      FMC_PHASE_SYNC(B, 11);
    }
    if (threadIdx.x == 32) run_deferred<F32, GN>(B);
    __syncthreads();
  } else if (mode == kModeCreate) {
    for (int g = 0; g < B.S.ntpguest; ++g) {
      long long maxiter = 1000LL * B.S.g[g].insert0, iter = 0;
      while (B.H.nummols[g] < B.S.g[g].insert0) {
        if (iter >= maxiter) {  // insert_guests iteration cap (error 2320)
          st |= kStCapacity;
          break;
        }
        propose<F32, kTricOk<F32, GN>>(B, CA, chain, kPropInsert, g);
        evaluate_rare<F32, GN>(B, CA, chain, st);
        if (threadIdx.x == 0) B.mc.accepted = B.mc.overlap ? 0 : 1;
        __syncthreads();
        commit_rare(B, CA, chain, st);
        __syncthreads();
        ++iter;
      }
    }
  } else if (mode == kModeEval) {
    if (threadIdx.x == 0) B.mc = gctx[chain];
    __syncthreads();
    propose<F32, kTricOk<F32, GN>>(B, CA, chain, kPropExternal, 0);
    int full = 0;
    if (B.mc.kind != 0) full = evaluate_any<F32, GN>(B, CA, chain, st);
    if (threadIdx.x == 0) {
      B.mc.evaluated = 1;
      B.mc.accepted = 0;
      (void)full;
    }
  } else if (mode == kModeWidom) {
    double hsum = 0.0;
    long long nok = 0, ntot = 0;
    // one trial through the full evaluation (the block)
    auto full_trial = [&](int t) {
      if (threadIdx.x < 32) widom_propose(B, wj, t);
      __syncthreads();
      evaluate_any<F32, GN>(B, CA, chain, st);
      if (threadIdx.x == 0) {
        ++ntot;
        if (!B.mc.overlap) {  // H_const = exp(-estep / kboltz / temp), gcmc.f:2537-2541
          ++nok;
          hsum += exp(-1.0 * B.mc.estep / kKboltz / B.S.temp);
        }
        if (wj.estep_out) wj.estep_out[t] = B.mc.overlap ? 0.0 : B.mc.estep;
        if (wj.overlap_out) wj.overlap_out[t] = B.mc.overlap;
        // the energy probability grid of widom_grid's test insertions
        // (gcmc.f:2529-2532; not for positions given by the caller)
        if (!B.mc.overlap && !wj.xyz_in && CA.grid && B.S.prob_nsub > 0) {
          const double e = B.mc.estep;
          store_enprob(B, CA, chain, wj.iguest, &e);
        }
      }
      __syncthreads();
    };
    bool screened = false;
    if constexpr (F32 && !kTricOk<F32, GN>) screened = overlap_27(B.S);
    // Most test insertions end at the overlap test.  On the FP32 path with
    // 27-cell overlap tests, each warp first screens one trial against the
    // framework in float (widom_screen: a slot counts only when r^2 is
    // below the overlap distance squared by a margin well above the float
    // geometry's error), so a trial it marks overlapping overlaps in the
    // full test too; the others go through the full evaluation, in trial
    // order, so the Henry sum is the same every run.
    const GuestType &G = B.S.g[wj.iguest];
    const int ns = G.ns;
    if (threadIdx.x == 0) B.wsc.nscreened = 0;
    if (threadIdx.x < 9) B.wsc.cell[threadIdx.x] = (float)B.S.cell[threadIdx.x];
    if (threadIdx.x >= 32 && threadIdx.x < 32 + 3 * ns)
      B.wsc.tmpl[(threadIdx.x - 32) / 3][(threadIdx.x - 32) % 3] =
          (float)G.tmpl[(threadIdx.x - 32) / 3][(threadIdx.x - 32) % 3];
    __syncthreads();
    for (int c = 0; widom_trial(c, 0, 0) < wj.ntrial; ++c) {  // chunks of kScreenPer rounds
      if (screened) {
        widom_screen(B, wj, c);
      } else if ((threadIdx.x & 31) == 0) {
        for (int kk = 0; kk < kScreenPer; ++kk) {
          const long long t = widom_trial(c, kk, threadIdx.x >> 5);
          B.wsc.list[kk][threadIdx.x >> 5] = t < wj.ntrial ? (int)t : -1;
        }
      }
      __syncthreads();
      for (int kk = 0; kk < kScreenPer; ++kk)
        for (int q = 0; q < kWarps; ++q) {
          const int tq = B.wsc.list[kk][q];
          if (tq >= 0) full_trial(tq);
        }
      __syncthreads();
    }
    if (threadIdx.x == 0) ntot += B.wsc.nscreened;
    if (threadIdx.x == 0) {
      wj.partial[3 * blockIdx.x] = hsum;
      wj.partial[3 * blockIdx.x + 1] = (double)nok;
      wj.partial[3 * blockIdx.x + 2] = (double)ntot;
    }
  } else if (mode == kModeLoad) {
    // molecules read from a restart file, in order: each inserted where it
    // is, whatever it overlaps (revread loads them as they are), and
    // committed with the energy changes of every molecule type
    for (int t = 0; t < wj.ntrial; ++t) {
      if (threadIdx.x < 32) widom_propose(B, wj, t);
      if (threadIdx.x == 0) {
        B.flags[4] = 0;
        B.flags[6] = 1;  // no overlap test
      }
      __syncthreads();
      evaluate_rare<F32, GN>(B, CA, chain, st);
      if (threadIdx.x == 0) B.mc.accepted = 1;
      __syncthreads();
      commit_rare(B, CA, chain, st);
      __syncthreads();
    }
  } else if (mode == kModeCommit) {
    // nmoves carries the host's decision (0 or 1), or -1 for energy_eval
    // on the device with the rande in gctx
    if (threadIdx.x == 0) {
      B.mc = gctx[chain];
      if (B.mc.forced) B.mc.accepted = B.mc.overlap ? 0 : 1;  // accept_move called directly
      else if (nmoves >= 0) B.mc.accepted = nmoves;
      else decide(B, false);
    }
    __syncthreads();
    if constexpr (F32) {
      // the evaluated position as the evaluation split it (FP64 positions
      // of the per-move ABI into hi/lo pairs): commit stores these
      if (threadIdx.x < 3 * B.mc.ns) {
        const int s = threadIdx.x / 3, d = threadIdx.x % 3;
        const double v = B.mc.pos[0][s][d];
        const float h = (float)v;
        B.ev.phi[0][s][d] = h;
        B.ev.plo[0][s][d] = (float)(v - (double)h);
      }
      __syncthreads();
    }
    commit(B, CA, chain, st);
    if (threadIdx.x == 0) B.mc.evaluated = 0;
  }
  if (st) atomicOr(&B.flags[0], st);
  __syncthreads();
  if (csize > 1) {
    cluster_barrier();  // every CTA's status is final
    if (rank == 0 && threadIdx.x == 0)
      for (int q = 1; q < csize; ++q) B.flags[0] |= dsmem_load_s32(dsmem_addr(&B.flags[0], q));
    cluster_barrier();  // the peers stay resident until rank 0 has read them
  }
  if (mode == kModeWidom) {  // read-only: the chain's state is left as it was
    if (st) wj.partial[3 * blockIdx.x + 2] = -1.0;  // flags a device status to the host
    return;
  }
  if (F32 && CA.resident && rank == 0) {
    // write the guests back in molecule order: molecule i in slot i
    const int n = B.H.nummols[0], ns = B.S.g[0].ns;
    const size_t base = (size_t)chain * kMaxG * CA.cap * kMaxS;
    int *ord = CA.ord + (size_t)chain * kMaxG * CA.cap;
    for (int idx = threadIdx.x; idx < n * ns; idx += kThreads) {
      const int i = idx / ns, sidx = idx - i * ns;
      const size_t o = base + (size_t)i * kMaxS + sidx;
      const float4 h = B.grh[idx], l = B.grl[idx];
      CA.ghi[o] = h;
      CA.glo[o] = l;
      CA.gpos[o * 3] = (double)h.x + (double)l.x;
      CA.gpos[o * 3 + 1] = (double)h.y + (double)l.y;
      CA.gpos[o * 3 + 2] = (double)h.z + (double)l.z;
    }
    for (int i = threadIdx.x; i < n; i += kThreads) ord[i] = i;
    if (threadIdx.x == 0) {
      B.H.nslots[0] = n;
      B.H.nfree[0] = 0;
    }
  }
  if (threadIdx.x == 0) {
    B.H.status |= B.flags[0];
    B.H.dev_ns += (long long)(global_ns() - t_start);
    if ((mode == kModeEval || mode == kModeCommit) && rank == 0) {
      B.mc.dev_status = B.H.status;  // read back with the move: no separate status read
      gctx[chain] = B.mc;
    }
  }
  __syncthreads();
  if (rank == 0) block_copy(hdrs + chain, &B.H);
}


// Launch and set-up of one instantiation, for the host side of the library.
// `nchains` chains (ids in chain_ids, or 0..nchains-1 when null), each on a
// cluster of csize CTAs.
template <bool F32, int GN>
cudaError_t launch_chain(int nchains, int csize, const int *chain_ids, size_t smem,
                         cudaStream_t stream, const SysDev *systems, ChainHdr *hdrs,
                         const ChainArrays &CA, MoveCtx *gctx, LogRec *logs, int logcap,
                         int nmoves, int mode, const double *ctl_fuga, const WidomJob &wj) {
  if (csize == 1) {
    chain_kernel<F32, GN><<<nchains, kThreads, smem, stream>>>(
        systems, hdrs, CA, gctx, logs, logcap, nmoves, mode, ctl_fuga, chain_ids, 1, wj);
    return cudaGetLastError();
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(nchains * csize));
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, chain_kernel<F32, GN>, systems, hdrs, CA, gctx, logs, logcap,
                            nmoves, mode, ctl_fuga, chain_ids, csize, wj);
}

// Clusters of csize CTAs that can be resident at once (0: cannot launch).
template <bool F32, int GN>
cudaError_t max_clusters(int csize, size_t smem, int *out) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)csize);
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaOccupancyMaxActiveClusters(out, chain_kernel<F32, GN>, &cfg);
}

template <bool F32, int GN>
cudaError_t set_chain_smem(size_t smem) {
  return cudaFuncSetAttribute(chain_kernel<F32, GN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)smem);
}

}  // namespace fmc

// device_core.cuh -- device data structures and the cooperative (one CTA)
// trial-move energy evaluation for sm_103a.
//
// Layout in HBM (all L2-resident for the benchmark sizes):
//  * framework atoms sorted by cell, z fastest: FP64 (x,y,z,q) records for
//    the FP64 path, and FP32 hi/lo pairs (x_hi,y_hi,z_hi,q)+(x_lo,y_lo,z_lo,-)
//    for the FP32 path, so that r = |p - a| keeps ~1 ulp of FP32 relative
//    accuracy even at 100 A coordinates;
//  * k-vectors in the reference order (ewald.f:151-315) as (l,m,n) and a_k;
//  * per chain: guest site coordinates by slot, the molecule order the
//    reference keeps (molxxx, mc_moves.f:574-590) as a slot list, the FP64
//    structure factor of each guest type, FP32 mirrors of S(k) and the s(k)
//    scratch of the last evaluation (the reference's ckcsnew/ckssnew).
//
// One CTA evaluates one guest position: the framework part scans the cell
// columns that intersect the sphere of radius rc + r_mol around the
// molecule (load-balanced over the CTA through a prefix sum of the column
// segments), the guest part loops over guest molecules, and the k-space
// part gives each thread a strided set of k-vectors with per-site power
// tables e^{i 2 pi j s_d} in shared memory.  Reductions are fixed-order
// warp-shuffle trees, so results are bitwise reproducible.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fmcdev {

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxS = 8;    // sites per guest
constexpr int kMaxG = 4;    // guest types
constexpr int kMaxProbItems = 32;  // probability-grid (subgrid, site) items per system
constexpr int kMaxM = 8;    // molecule types
constexpr int kMaxT = 16;   // atom types
constexpr int kMaxKm = 40;  // kmax per axis + 1
constexpr int kPlmMax = 4352;  // entries of the FP32 (l, m) phase table (34 KB)
constexpr int kMaxSeg = 1024;

// status word bits (ChainHdr::status)
constexpr int kStTableLow = 1;     // pair closer than one grid step
constexpr int kStSegOverflow = 2;  // too many framework segments
constexpr int kStCapacity = 4;     // guest capacity exceeded
constexpr int kStNonFinite = 8;    // non-finite energy
constexpr int kStBadChoice = 16;   // molecule index out of range
constexpr int kStKmax = 32;        // kmax beyond the shared tables
constexpr int kStWait = 64;        // a bounded wait on an asynchronous copy ran out
constexpr int kStDraws = 128;      // generator buffer empty (internal error)
constexpr int kStIndex = 256;      // a guest slot or position out of range (access skipped)
constexpr int kRBuf = 256;         // generator outputs drawn ahead per chain (power of two)

constexpr double kPi = 3.141592653589793;
constexpr double kSqrPi = 1.7724538509055159;
constexpr double kR4pie0 = 138935.4835;
constexpr double kBoltz = 1.3806503e-23;  // J/K (boltz, utility_pack.f:124)
constexpr double kKboltz = 1.9872041e-3;  // kcal/mol/K (kboltz, utility_pack.f:121)
constexpr double kRgas = 8.314472 / 4184.0;
constexpr double kMinAngle = kPi / 18.0;
constexpr double kDelrMin = 0.1;

// ----------------------------------------------------------------- params
struct GuestType {
  int mol;        // molecule type (1-based)
  int ns;         // sites
  float rns;      // 1 / ns
  int insert0;    // "create molecules"
  int pad;
  double q[kMaxS];
  double mass[kMaxS];
  double tmpl[kMaxS][3];   // centred template (readinputs.f:221-243)
  int type[kMaxS];         // atom type 1..ntpatm
  int frz[kMaxS];
  double ewald3en;
  double chgea[kMaxS];     // q / epsq * r4pie0 per site (ewald2's charge factor)
  float tmplf[kMaxS][3];   // centred template in FP32 (FP32 trial geometry)
  float tmplf_lo[kMaxS][3];  // template - tmplf (double-float trial geometry)
  int prow[kMaxS][kMaxT + 1];      // table row of site s with atom type t (-1: none)
  float psig2[kMaxS][kMaxT + 1];   // (surftol + sigma)^2 of site s with atom type t
  float wf[kMaxS];         // mass fraction of each site (centre of mass)
  float wf_lo[kMaxS];      // mass fraction - wf
  float chgeaf[kMaxS];     // the same as an FP32 hi/lo pair
  float chgeaf_lo[kMaxS];
  // constants of the energy expressions of this guest type
  double chgtmp;           // sum of site charges
  double engsic0;          // self-interaction -r4pie0/epsq*alpha*sum(q^2)/sqrt(pi)
  double qfa, qfb;         // charged-system term qfix = qfa*sumchg + qfb
  double qfm;              // qfixmol(m) = qfm * chgsum_mol(m)
  double rmass;            // 1 / molecular mass (com)
  // LJ long-range tail of one molecule (gstlrcorrect) as a linear function
  // of the guest counts: insert lrcA + sum_g2 N_g2 lrcB[g2];
  // delete -lrcA + 2 lrcC - sum_g2 N_g2 lrcB[g2]; framework part lrcA - lrcC
  double lrcA, lrcC, lrcB[kMaxG];
  double rmax;             // max site distance from the template centre
  double delr;             // displacement size / list skin
  double disp_ratio, tran_ratio, rota_ratio;
  float mcinsf, mcdelf, mcdisf, mcjmpf, mcswpf, mctraf, mcrotf, mcswif;
};

// Per-system data, shared by every chain that uses the system.
struct SysDev {
  // cell
  int imcon;
  double cell[9], rcell[9], box[3];
  double volm, statvolm, temp, beta, engunit, rengunit, epsq, alpha;
  double rcut, rc2, overlap_sq, surftol;
  double sumchg0;          // system charge without guests
  double chgsum_fw;        // framework charge (chgsum_mol of the framework)
  int maxmls, ntpguest, ntpatm, fw_mol;
  int eqsteps, nwindsteps, minchk, laccsample;
  // framework
  int nfw;
  const double4 *fw64;     // x,y,z,q (wrapped into the cell for imcon 1/2)
  const float4 *fwhi;      // x_hi,y_hi,z_hi,q
  const float4 *fwlo;      // x_lo,y_lo,z_lo,0
  const int *fwtype;
  int use_cells;
  int nc[3];
  double csz[3];
  double rcsz[3];          // 1 / csz
  double rbox[3];          // 1 / L, the reference's aaa = 1/cell (images)
  float boxh[3], boxl[3];  // L as a float hi/lo pair
  // parallelepiped cells (imcon 3), FP32 path: cell and its inverse as
  // float hi/lo pairs, the reference's layout (cell[0..2] the first edge)
  float cellh[9], celll[9], rcellh[9], rcelll[9];
  float rboxf[3], rcszf[3], cszf[3];
  float rboxf_lo[3];       // 1/L - rboxf
  float overlap_sqf, rc2f, rdrewdf, rdlrpotf;
  float rdlrpotf_lo;       // rdlrpot - rdlrpotf (double-float bin index of close pairs)
  const int *cell_start;   // [nc0*nc1*nc2+1], z fastest
  // the same cells padded to 2^cpad_log2 slots (empty slots far away):
  // the overlap test reads a cell's atoms without reading cell_start first
  int cpad_log2;
  const float4 *cpad_hi, *cpad_lo;
  // tables
  int mxegrd;
  double rdrewd, rdlrpot;
  const double *erc;       // [mxegrd+3], 1-based
  const double *vvv;       // [ntab][mxegrd+3]
  const float4 *ercq;      // per interval (A,B,C,A_lo): value = A + p(B + pC), A_lo = v0 - A
  const float4 *vvvq;      // [ntab][mxegrd+3]
  int tabstride;           // mxegrd+3
  const int *pairtab;      // [(ntpatm+1)^2] -> table row or -1
  const double *sig2;      // [(ntpatm+1)^2] (surftol + sigma)^2
  const float *sig2f;
  const double *steadd;    // [loc2 pair] tail constants
  const int *numtyp_fw, *numfrz_fw;   // [ntpatm+1]
  // k-space
  int nk, kmax[3];
  const int4 *klmn;        // (l,m,n,0)
  const unsigned *kpk;     // l * (2 kmax_y + 1) + m + kmax_y | (n + 128) << 16
  const double *akk;
  const float *akk32;
  const double2 *skfw;     // framework S(k)
  const float4 *skfw_df;   // framework S(k) as FP32 hi/lo pairs (re_hi, im_hi, re_lo, im_lo)
  double krecip;           // 2 * rvolm * r4pie0 / epsq
  // probability grids (storeprob): per guest type, items (subgrid, site)
  // binned for every molecule after each production move
  int prob_nsub, prob_gridsize;
  int ngrid[3];
  double rucell[9];        // inverse of the unit (folding) cell
  int prob_nitem[kMaxG], prob_item0[kMaxG];
  int prob_eng_sub[kMaxG];         // energy grids: the energy-sum subgrid (the count is the
                                   // next one), -1 without
  short prob_sub[kMaxProbItems];   // 0-based subgrid
  short prob_site[kMaxProbItems];  // 0: centre of mass, else 1-based site
  // guests
  GuestType g[kMaxG];
};

// Per-chain scalar state (one record per chain in global memory).
struct ChainHdr {
  float u[97];
  float c, cd, cm;
  int ir, jr;
  int nummols[kMaxG];
  int nslots[kMaxG];       // high-water mark of slots
  int nfree[kMaxG];
  int status;
  double energy[kMaxM + 1];      // energy(mol), 1-based
  double chgsum_mol[kMaxM + 1];
  double sumchg;
  double surfacemols[kMaxM + 1];
  int numtyp[kMaxT + 1], numfrz[kMaxT + 1];
  int numtyp_mol[kMaxM + 1][kMaxT + 1];
  int numfrz_mol[kMaxM + 1][kMaxT + 1];
  double delrdisp[kMaxG], tran_delr[kMaxG];
  double rotangle, rota_rotangle;
  double fuga[kMaxG];
  long long ins_count[kMaxG], accept_ins[kMaxG], del_count[kMaxG], accept_del[kMaxG];
  long long disp_count[kMaxG], accept_disp[kMaxG], tran_count[kMaxG], accept_tran[kMaxG];
  long long rota_count[kMaxG], accept_rota[kMaxG];
  long long jump_count[kMaxG], accept_jump[kMaxG];
  long long gcmccount, prodcount, rollcount;
  int production;
  int minchk_left;         // moves until gcmccount is next a multiple of minchk
  int window_left;         // production moves until the next window ends
  int last_accepted;       // the previous move's decision (a switch no-op keeps it)
  long long pend;          // production moves not yet added to chainstats (FP32 path)
  long long dev_ns;        // device time spent in this chain's launches (ns)
  double chainstats[kMaxG][6];
  double wsum;
  double wacc[kMaxG][8];
  double wsq[kMaxG];       // sum over windows of weight x <N>_window^2 (standard error)
  long long windows;
  long long moves, evals, overlap_exits;
  long long attempts[8], accepts[8];  // insert, delete, displace, translate, rotate, jump, swap, switch
  long long log_n;
  int system;
  int pad1;
  // FP32 path: the step sizes as float hi/lo pairs, kept equal to the
  // doubles above (sync_step_pairs after every change)
  float sh_disp[kMaxG][2];  // 0.5 * delrdisp
  float sh_tran[kMaxG][2];  // 0.5 * tran_delr
  float rho_rot[2][2];      // rotangle / (2 pi), rota_rotangle / (2 pi)
  // generator outputs drawn ahead (refill_draws), consumed in order
  float rbuf[kRBuf];
  int rhead, ravail;
  // disp_count, tran_count, rota_count modulo 100 (the adaptive-step tests)
  int disp_mod[kMaxG], tran_mod[kMaxG], rota_mod[kMaxG];
  float lnpf[kMaxG];  // FP32 decisions: log(statvolm * fugacity / (kB T)), per launch
  int skb[kMaxG];     // FP32 path: guest S(k) of type g is in skdf (0) or skdf2 (1)
  long long phase_cycles[16];  // move-loop clocks per phase (FMC_PHASE_TIMERS builds)
};

__host__ __device__ inline void split_pair(double x, float *out) {
  out[0] = (float)x;
  out[1] = (float)(x - (double)out[0]);
}

// The pairs of guest type g and the two rotation angles.
__host__ __device__ inline void sync_step_pairs(ChainHdr &h, int g) {
  split_pair(0.5 * h.delrdisp[g], h.sh_disp[g]);
  split_pair(0.5 * h.tran_delr[g], h.sh_tran[g]);
  split_pair(h.rotangle * (0.5 / kPi), h.rho_rot[0]);
  split_pair(h.rota_rotangle * (0.5 / kPi), h.rho_rot[1]);
}

// Per-chain arrays.
struct ChainArrays {
  double *gpos;     // [chain][g][slot][site] x,y,z (stride 3)
  float4 *ghi;      // [chain][g][slot][site] hi mirror (x,y,z,q)
  float4 *glo;      // [chain][g][slot][site] lo mirror
  int *ord;         // [chain][g][cap] slot ids in molecule order
  int *freel;       // [chain][g][cap]
  double2 *sk;      // [chain][g][nkmax] guest S(k), FP64 path
  float4 *skdf;     // [chain][g][nkmax] guest S(k) as FP32 hi/lo pairs, FP32 path
  float4 *skdf2;    // the second buffer: an evaluation writes the updated S(k)
                    // there and an accepted move flips ChainHdr::skb
  double2 *snew;    // [chain][nkmax] scratch s(k) of the evaluated position
  double2 *sold;    // [chain][nkmax] scratch s(k) of the old position
  double2 *sksave;  // [chain][2][nkmax] FP64 path, systems with swap moves: the two
                    // guest types' S(k) before a swap, for its rejection (else null)
  const float4 *trig;  // [kTrigN] sin(2 pi k/kTrigN) hi, lo, cos(2 pi k/kTrigN) hi, lo
  double *grid;        // [chain][subgrid][bin] probability grids (null: none)
  size_t grid_stride;  // doubles per chain
  int cap;          // molecules per guest type
  int nkmax;
  int resident;     // FP32 batches of one guest type: guests held in shared memory
  int spec_max;     // proposals per speculative round at most (below 2: none)
};

// Entries of the sine/cosine table of the double-float quaternions (one
// turn): half angles pi * rho are split at the nearest multiple of
// 2 pi / kTrigN.
constexpr int kTrigN = 128;

// Guest sites a CTA can hold in shared memory (molecule order, hi/lo).
constexpr int kGuestSmem = 3072;

// Widom test insertions against one chain's current state (widom_grid,
// gcmc.f:2454-2548): trial t is grid point t / nstep (fractions i/ng0,
// j/ng1, k/ng2, 1-based as the reference loops) with a random orientation,
// or the given site coordinates xyz_in[t].  Per CTA: sum of
// exp(-estep/(kB T)) over non-overlapping trials, their count, all trials.
struct WidomJob {
  int chain, iguest;       // chain index, guest type (0-based)
  int ntrial, nstep;
  int ng[3];
  int pad;
  unsigned long long seed;
  const double *xyz_in;    // [ntrial][ns][3] or null
  double *estep_out;       // [ntrial] or null (0 for an overlap)
  int *overlap_out;        // [ntrial] or null
  double *xyz_out;         // [ntrial][ns][3] or null
  double *partial;         // [gridDim.x][3]
};

// Counter-based uniform variate in [0, 1) with 24 bits, like the
// generator's values: the splitmix64 finaliser of (seed, index).
__host__ __device__ inline float hash_uniform(unsigned long long seed, unsigned long long i) {
  unsigned long long z = seed + 0x9e3779b97f4a7c15ULL * (i + 1);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  z ^= z >> 31;
  return (float)(z >> 40) * (1.0f / 16777216.0f);
}

// Description of one trial move (shared memory; copied to global between
// the evaluate and commit kernels of the per-move ABI).
struct MoveCtx {
  int kind;           // 1 insert, 2 delete, 3 displace, 4 translate, 5 rotate
  int g;              // guest type, 0-based
  int choice;         // 1-based molecule (delete / displace)
  int slot;           // storage slot of the molecule
  int ns;
  int overlap;
  int surf_new, surf_old;
  int accepted;
  int evaluated;
  int npos;           // 1 or 2 positions evaluated
  int forced;         // commit mode: accept without a decision (a swap's halves)
  int dev_status;     // per-move ABI: the chain's status word after the launch
  double pos[2][kMaxS][3];   // [0] = new / inserted / deleted, [1] = old (displace)
  double estep;
  double rande;
  double delrc;
  double delE[kMaxM + 1];
  double delrc_mol[kMaxM + 1];
  double parts[4];           // ewld1, ewld2, vdw, delrc of position 0
  double ewld1_b;
  double chgtmp, engsictmp;
};

struct Acc {  // per-position partial sums
  double e2_fw, vdw_fw;
  double e2_g[kMaxG], vdw_g[kMaxG];
  double recip;
  double mix[kMaxM + 1];
};

// ------------------------------------------------- padding, waits
constexpr int kKT = kThreads;       // k-vector arrays are padded to multiples of this
constexpr int kWaitLimit = 1 << 22; // polls before a bounded wait gives up

__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

// ------------------------------------------------- thread-block clusters
// A chain may run on a cluster of up to kMaxCluster CTAs.  Exchanges between
// them go through distributed shared memory: release/acquire flag stores
// into the peers' shared memory and bounded polling of one's own flags.
constexpr int kMaxCluster = 8;

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
// Every thread of every CTA of the cluster (unconditional call sites only).
__device__ __forceinline__ void cluster_barrier() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::
                   : "memory");
}
// Shared-memory address of the same variable in CTA `rank` of the cluster.
__device__ __forceinline__ unsigned dsmem_addr(const void *p, unsigned rank) {
  unsigned r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
  return r;
}
__device__ __forceinline__ void dsmem_store_release(unsigned addr, unsigned v) {
  asm volatile("st.release.cluster.shared::cluster.u32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned dsmem_load_acquire(unsigned addr) {
  unsigned v;
  asm volatile("ld.acquire.cluster.shared::cluster.u32 %0, [%1];" : "=r"(v) : "r"(addr) : "memory");
  return v;
}
__device__ __forceinline__ double dsmem_load_f64(unsigned addr) {
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(addr) : "memory");
  return v;
}
__device__ __forceinline__ int dsmem_load_s32(unsigned addr) {
  int v;
  asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(addr) : "memory");
  return v;
}
// Poll one's own flag until it reaches `seq`; false if it did not in time.
__device__ __forceinline__ bool wait_flag(const unsigned *flag, unsigned seq) {
  const unsigned a = smem_u32(flag);
  for (int it = 0; it < kWaitLimit; ++it)
    if ((int)(dsmem_load_acquire(a) - seq) >= 0) return true;
  return false;
}
// [lo, hi) of `n` items for member `r` of `c`.
__device__ __forceinline__ void share_of(int n, int r, int c, int &lo, int &hi) {
  lo = (int)(((long long)n * r) / c);
  hi = (int)(((long long)n * (r + 1)) / c);
}

// ----------------------------------------------------------- MZT generator
// duni (utility_pack.f:2768-2857): REAL*4 lagged subtract-with-borrow plus
// a Weyl term; one step: uni = u[ir] - u[jr] (+1 if negative), u[ir] = uni,
// ir and jr step down cyclically (97 -> 1), c -= cd (+cm if negative),
// output uni - c (+1 if negative).  Bit-exact because only float
// add/sub/compare of multiples of 2^-24 are used.

// The generator run ahead by one warp: 32 consecutive outputs per
// call, one per lane, appended to the chain's buffer.  duni's state update
// is x_t = x_{t-97} - x_{t-33} (mod 1) on u[] and c_t = c_{t-1} - cd
// (mod cm); within 32 steps a lane reads u[] entries no other lane writes
// (the read of step t at offset 33 lies before the batch, the writes of the
// batch are its own positions), and c after k steps is (c - k cd) mod cm in
// exact units of 2^-24.  Outputs are bit-identical to 32 sequential steps.
__device__ __forceinline__ void refill_draws(ChainHdr &h) {
  const int lane = threadIdx.x & 31;
  const int ir0 = h.ir, jr0 = h.jr;
  int ir = ir0 - 1 - lane, jr = jr0 - 1 - lane;
  if (ir < 0) ir += 97;
  if (jr < 0) jr += 97;
  float uni = h.u[ir] - h.u[jr];
  if (uni < 0.0f) uni += 1.0f;
  const int C0 = (int)(h.c * 16777216.0f), CD = (int)(h.cd * 16777216.0f),
            CM = (int)(h.cm * 16777216.0f);
  int ci = (C0 - (lane + 1) * CD) % CM;
  if (ci < 0) ci += CM;
  const float c = (float)ci * (1.0f / 16777216.0f);
  float out = uni - c;
  if (out < 0.0f) out += 1.0f;
  const int pos = (h.rhead + h.ravail + lane) & (kRBuf - 1);
  __syncwarp();
  h.u[ir] = uni;
  h.rbuf[pos] = out;
  __syncwarp();
  if (lane == 31) h.c = c;
  if (lane == 0) {
    h.ir = ir0 - 32 > 0 ? ir0 - 32 : ir0 - 32 + 97;
    h.jr = jr0 - 32 > 0 ? jr0 - 32 : jr0 - 32 + 97;
    h.ravail += 32;
  }
  __syncwarp();
}

// Next generator output (lane 0 of warp 0; the buffer holds at least one
// move's draws, refilled at the start of every proposal).
__device__ __forceinline__ float draw_f(ChainHdr &h) {
  if (h.ravail <= 0) {
    h.status |= kStDraws;
    return 0.5f;
  }
  const float v = h.rbuf[h.rhead];
  h.rhead = (h.rhead + 1) & (kRBuf - 1);
  --h.ravail;
  return v;
}

// Several consecutive draws with the buffer position held in registers
// (the loads are independent); done() stores the position back.
struct DrawCursor {
  ChainHdr &h;
  int head, avail;
  __device__ __forceinline__ explicit DrawCursor(ChainHdr &hh) : h(hh), head(hh.rhead), avail(hh.ravail) {}
  __device__ __forceinline__ float next() {
    const float v = h.rbuf[head];
    head = (head + 1) & (kRBuf - 1);
    --avail;
    return v;
  }
  __device__ __forceinline__ void done() {
    if (avail < 0) h.status |= kStDraws;
    h.rhead = head;
    h.ravail = avail;
  }
};

// floor(u * n) + 1 for a generator value u (a multiple of 2^-24), exactly
// as the reference's floor(duni()*n)+1 in FP64 (gcmc.f:1782, 1870).
__device__ __forceinline__ int pick1(float u, int n) {
  unsigned long long m = (unsigned long long)(u * 16777216.0f);
  return (int)((m * (unsigned long long)n) >> 24) + 1;
}

// Initialisation from the clock values the reference reads
// (utility_pack.f:2796-2852).
__host__ __device__ inline void duni_init(ChainHdr &h, int ms, int sec) {
  int i = (ms * 3) % 177 + 1, j = (sec * 23) % 177 + 1, k = (ms * 5) % 177 + 1,
      l = (sec * 3) % 168;
  h.ir = 97;
  h.jr = 33;
  for (int ii = 0; ii < 97; ++ii) {
    float s = 0.0f, t = 0.5f;
    for (int jj = 0; jj < 24; ++jj) {
      int m = (((i * j) % 179) * k) % 179;
      i = j;
      j = k;
      k = m;
      l = (53 * l + 1) % 169;
      if ((l * m) % 64 >= 32) s = s + t;
      t = 0.5f * t;
    }
    h.u[ii] = s;
  }
  h.c = 362436.0f / 16777216.0f;
  h.cd = 7654321.0f / 16777216.0f;
  h.cm = 16777213.0f / 16777216.0f;
}

// ------------------------------------------------------------- geometry
__device__ __forceinline__ void cartesian(const SysDev &S, double a, double b,
                                          double c, double *o) {
  o[0] = a * S.cell[0] + b * S.cell[3] + c * S.cell[6];
  o[1] = a * S.cell[1] + b * S.cell[4] + c * S.cell[7];
  o[2] = a * S.cell[2] + b * S.cell[5] + c * S.cell[8];
}

// rotation (utility_pack.f:3480-3524)
__device__ inline void rotate_sites(double (*p)[3], int n, const double *cm,
                                    double q1, double q2, double q3, double q4) {
  double Q[9];
  Q[0] = 2.0 * q2 * q2 + 2.0 * q1 * q1 - 1.0;
  Q[1] = 2.0 * q2 * q3 - 2.0 * q1 * q4;
  Q[2] = 2.0 * q2 * q4 + 2.0 * q1 * q3;
  Q[3] = 2.0 * q2 * q3 + 2.0 * q1 * q4;
  Q[4] = 2.0 * q1 * q1 + 2.0 * q3 * q3 - 1.0;
  Q[5] = 2.0 * q3 * q4 - 2.0 * q1 * q2;
  Q[6] = 2.0 * q2 * q4 - 2.0 * q1 * q3;
  Q[7] = 2.0 * q3 * q4 + 2.0 * q1 * q2;
  Q[8] = 2.0 * q4 * q4 + 2.0 * q1 * q1 - 1.0;
  for (int i = 0; i < n; ++i) {
    double x = p[i][0] - cm[0], y = p[i][1] - cm[1], z = p[i][2] - cm[2];
    double tx = Q[0] * x + Q[1] * y + Q[2] * z;
    double ty = Q[3] * x + Q[4] * y + Q[5] * z;
    double tz = Q[6] * x + Q[7] * y + Q[8] * z;
    p[i][0] = tx + cm[0];
    p[i][1] = ty + cm[1];
    p[i][2] = tz + cm[2];
  }
}

// com (utility_pack.f:3565-3596)
__device__ inline void centre_of_mass(const GuestType &G, double (*p)[3],
                                      double *cm) {
  double w = 0.0;
  cm[0] = cm[1] = cm[2] = 0.0;
  for (int i = 0; i < G.ns; ++i) {
    w += G.mass[i];
    cm[0] += p[i][0] * G.mass[i];
    cm[1] += p[i][1] * G.mass[i];
    cm[2] += p[i][2] * G.mass[i];
  }
  cm[0] /= w;
  cm[1] /= w;
  cm[2] /= w;
}

// random quaternion of random_ins / random_rot (utility_pack.f:3266-3330,
// 3526-3563): theta = rand1 * angle, axis from three uniforms.
__device__ inline void quaternion(double r1, double r2, double r3, double r4,
                                  double angle, double *q) {
  double theta = r1 * angle;
  double b1 = 2.0 * r2 - 1.0, b2 = 2.0 * r3 - 1.0, b3 = 2.0 * r4 - 1.0;
  double st = sin(theta / 2.0);
  double nrm = sqrt(b1 * b1 + b2 * b2 + b3 * b3);
  q[0] = cos(theta / 2.0);
  q[1] = st * (b1 / nrm);
  q[2] = st * (b2 / nrm);
  q[3] = st * (b3 / nrm);
}

// translate (utility_pack.f:3161-3218)
__device__ inline void translate_sites(const SysDev &S, const GuestType &G,
                                       double (*p)[3], double a, double b,
                                       double c) {
  for (int i = 0; i < G.ns; ++i) {
    p[i][0] = a + p[i][0];
    p[i][1] = b + p[i][1];
    p[i][2] = c + p[i][2];
  }
  double cm[3];
  centre_of_mass(G, p, cm);
  const double *r = S.rcell;
  double sx = r[0] * cm[0] + r[3] * cm[1] + r[6] * cm[2];
  double sy = r[1] * cm[0] + r[4] * cm[1] + r[7] * cm[2];
  double sz = r[2] * cm[0] + r[5] * cm[1] + r[8] * cm[2];
  sx -= floor(sx);
  sy -= floor(sy);
  sz -= floor(sz);
  double w[3];
  cartesian(S, sx, sy, sz, w);
  double d0 = w[0] - cm[0], d1 = w[1] - cm[1], d2 = w[2] - cm[2];
  for (int i = 0; i < G.ns; ++i) {
    p[i][0] += d0;
    p[i][1] += d1;
    p[i][2] += d2;
  }
}

// ------------------------------------------------------------ reductions
template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Fixed-order block sum of n values per thread; result valid in red[0..n).
__device__ inline void block_sum(double *vals, int n, double *red) {
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = 0; i < n; ++i) {
    double v = warp_sum(vals[i]);
    if (lane == 0) red[w * n + i] = v;
  }
  __syncthreads();
  if (threadIdx.x < n) {
    double s = 0.0;
    for (int k = 0; k < kWarps; ++k) s += red[k * n + threadIdx.x];
    red[kWarps * n + threadIdx.x] = s;
  }
  __syncthreads();
}

__device__ inline int block_or(int v, int *scratch) {
  (void)scratch;
  return __syncthreads_or(v) ? 1 : 0;  // one barrier that also reduces
}

// Exclusive block scan of one int per thread; returns the total.
__device__ inline int block_scan(int v, int &excl, int *scratch) {
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) scratch[w] = x;
  __syncthreads();
  int base = 0, tot = 0;
  for (int k = 0; k < kWarps; ++k) {
    if (k < w) base += scratch[k];
    tot += scratch[k];
  }
  excl = base + x - v;
  __syncthreads();
  return tot;
}

// ------------------------------------------- error-free FP32 arithmetic
// A value held as an unevaluated sum hi + lo of two floats (about 48
// significant bits).  Used for the FP32 path's accumulators and for its
// running structure factor, so no FP64 instruction is needed there.
// rint(x) for the minimum image of two points in or near one cell: with
// |x| < 1.5 the result is -1, 0 or 1 (ties to even as rint: 0 at +-1/2),
// taken by comparisons; a rounding instruction only otherwise (those issue
// to the FP64 pipe, narrow on this part, and sit on the pair's dependency
// chain).  The same value as rintf(x) except for the sign of a zero.
__device__ __forceinline__ float rint_image(float x) {
  if (fabsf(x) < 1.5f) return (x > 0.5f ? 1.f : 0.f) - (x < -0.5f ? 1.f : 0.f);
  return rintf(x);
}

__device__ __forceinline__ void two_sum_f(float a, float b, float &s, float &e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

struct DF {
  float hi, lo;
  __device__ __forceinline__ void add(float x) {
    float s, e;
    two_sum_f(hi, x, s, e);
    hi = s;
    lo += e;
  }
  __device__ __forceinline__ void add(DF o) {
    float s, e;
    two_sum_f(hi, o.hi, s, e);
    e += lo + o.lo;
    hi = s + e;
    lo = e - (hi - s);
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// Double-float values for the FP32 path's trial geometry: h + l with
// |l| <= ulp(h)/2.  Products use __fmul_rn and explicit fmaf so that no
// product is contracted into a following sum (which would break the
// error-free steps).  Sums: two_sum of the high parts, low parts added,
// renormalised; products: exact high product by fmaf plus cross terms.
struct F2 {
  float h, l;
};
__device__ __forceinline__ F2 f2_norm(float a, float b) {  // |a| >= |b| or a == 0
  const float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
  float s, e;
  two_sum_f(a.h, b.h, s, e);
  e += a.l + b.l;
  return f2_norm(s, e);
}
__device__ __forceinline__ F2 f2_addf(F2 a, float b) {
  float s, e;
  two_sum_f(a.h, b, s, e);
  return f2_norm(s, e + a.l);
}
__device__ __forceinline__ F2 f2_neg(F2 a) { return {-a.h, -a.l}; }
__device__ __forceinline__ F2 f2_sub(F2 a, F2 b) { return f2_add(a, f2_neg(b)); }
__device__ __forceinline__ F2 f2_mul(F2 a, F2 b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return f2_norm(p, e);
}
__device__ __forceinline__ F2 f2_mulf(F2 a, float b) {
  const float p = __fmul_rn(a.h, b);
  float e = fmaf(a.h, b, -p);
  e = fmaf(a.l, b, e);
  return f2_norm(p, e);
}
__device__ __forceinline__ F2 f2_shfl(F2 a, int src) {
  return {__shfl_sync(0xffffffffu, a.h, src), __shfl_sync(0xffffffffu, a.l, src)};
}

template <bool F32>
struct AccT;
template <>
struct AccT<false> {
  double v;
  __device__ __forceinline__ void zero() { v = 0.0; }
  __device__ __forceinline__ void add(double x) { v += x; }
};
template <>
struct AccT<true> {
  DF v;
  __device__ __forceinline__ void zero() { v.hi = v.lo = 0.f; }
  __device__ __forceinline__ void add(float x) { v.add(x); }
  __device__ __forceinline__ void add_df(DF x) { v.add(x); }
};

// Per-position partial sums of one thread, for up to GN guest types.  The
// members are always addressed with compile-time indices so the whole set
// stays in registers.
template <bool F32, int GN>
struct PosAcc {
  static constexpr int kN = 4 + 3 * GN;  // values per position
  AccT<F32> e2fw, vdwfw, recip, mixfw;
  AccT<F32> e2g[GN], vdwg[GN], mixg[GN];
  __device__ __forceinline__ void zero() {
    e2fw.zero();
    vdwfw.zero();
    recip.zero();
    mixfw.zero();
#pragma unroll
    for (int g = 0; g < GN; ++g) {
      e2g[g].zero();
      vdwg[g].zero();
      mixg[g].zero();
    }
  }
  // value j of the reduction layout: e2fw, vdwfw, recip, mixfw, e2g[GN],
  // vdwg[GN], mixg[GN]
  __device__ __forceinline__ const AccT<F32> &at(int j) const {
    if (j == 0) return e2fw;
    if (j == 1) return vdwfw;
    if (j == 2) return recip;
    if (j == 3) return mixfw;
    if (j < 4 + GN) return e2g[j - 4];
    if (j < 4 + 2 * GN) return vdwg[j - 4 - GN];
    return mixg[j - 4 - 2 * GN];
  }
};

__device__ __forceinline__ double warp_total(const AccT<false> &a) { return warp_sum(a.v); }
__device__ __forceinline__ DF warp_total(const AccT<true> &a) {
  DF x = a.v;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    DF y;
    y.hi = __shfl_xor_sync(0xffffffffu, x.hi, o);
    y.lo = __shfl_xor_sync(0xffffffffu, x.lo, o);
    x.add(y);
  }
  return x;
}

// Fixed-order block reduction of the partial sums of both positions:
// out[p * kN + j] = block total of value j of position p (as a double).
// Positions >= npos and guest types >= ng are skipped.
template <bool F32, int GN>
__device__ int block_reduce_pos(const PosAcc<F32, GN> &a0, const PosAcc<F32, GN> &a1, int npos,
                                int ng, double *scratch, double *out, int flags, int *iscratch) {
  constexpr int N = PosAcc<F32, GN>::kN;
  static_assert(2 * N <= 32, "reduction scratch holds 32 values per warp");
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  // OR of the per-thread flag bits rides on the same barriers
  const int wf = __reduce_or_sync(0xffffffffu, (unsigned)flags);
  if (lane == 0) iscratch[w] = wf;
#pragma unroll
  for (int i = 0; i < 2 * N; ++i) {
    const int p = i / N, j = i % N;
    if (p >= npos) continue;
    if (j >= 4 && (j - 4) % GN >= ng) continue;
    const auto x = warp_total(p == 0 ? a0.at(j) : a1.at(j));
    if (lane == 0) {
      if constexpr (F32) {
        float *sc = reinterpret_cast<float *>(scratch);
        sc[2 * (w * 32 + i)] = x.hi;
        sc[2 * (w * 32 + i) + 1] = x.lo;
      } else {
        scratch[w * 32 + i] = x;
      }
    }
  }
  __syncthreads();
  const int i = threadIdx.x;
  if (i < 2 * N) {
    const int p = i / N, j = i % N;
    double tot = 0.0;
    if (p < npos && !(j >= 4 && (j - 4) % GN >= ng)) {
      if constexpr (F32) {
        const float *sc = reinterpret_cast<const float *>(scratch);
        DF s;
        s.hi = s.lo = 0.f;
        for (int k = 0; k < kWarps; ++k) {
          DF y;
          y.hi = sc[2 * (k * 32 + i)];
          y.lo = sc[2 * (k * 32 + i) + 1];
          s.add(y);
        }
        tot = s.value();
      } else {
        for (int k = 0; k < kWarps; ++k) tot += scratch[k * 32 + i];
      }
    }
    out[i] = tot;
  }
  int r = 0;
  for (int k = 0; k < kWarps; ++k) r |= iscratch[k];
  __syncthreads();
  return r;
}

}  // namespace fmcdev

/*
 * fastmc_gb300.h -- C ABI of the GB300 (sm_103a) GCMC trial-move energy path.
 *
 * The ABI is plain C: opaque handles, pointers, sizes and int status codes
 * (0 = OK).  Every entry point is callable from Fortran through
 * ISO_C_BINDING (integer(c_int), real(c_double), type(c_ptr)).  Logical
 * flags are integer(c_int) 0/1.  Arrays are 0-based on this side; guest
 * type and molecule indices keep the reference's 1-based numbering.
 *
 * Three groups of entry points:
 *  1. Host set-up.  fmc_system_load reads FIELD, CONFIG and CONTROL and
 *     builds the tables and constants that the reference computes at start
 *     (gcmc.f:203-590) from the same input files the reference reads.
 *  2. Per-move drop-in ("plain" mode).  The device mirrors the host's
 *     guest coordinates and structure factor; each call evaluates one trial
 *     move and leaves s(k) on the device for the commit, exactly like
 *     ckcsnew/ckssnew in the reference.
 *  3. Device-resident chains ("batch" mode): many independent GCMC chains
 *     run their whole move loop on the device (RNG, proposal, energy,
 *     Metropolis, commit, statistics) in one persistent kernel per cycle.
 */
#ifndef FASTMC_GB300_H
#define FASTMC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes; a Fortran caller turns a positive value into a call of
 * the reference's error() routine with a code of its choosing */
#define FMC_OK 0
#define FMC_ERR_ARG 1      /* invalid argument or handle */
#define FMC_ERR_CUDA 2     /* CUDA runtime failure (message has details) */
#define FMC_ERR_CAPACITY 3 /* guest capacity or buffer size exceeded */
#define FMC_ERR_INPUT 4    /* malformed or unsupported input file content */
#define FMC_ERR_DEVICE 5   /* a kernel raised its status word (see message) */
#define FMC_ERR_STATE 6    /* call out of order (e.g. commit before a move) */
#define FMC_ERR_NODEVICE 7 /* no CUDA device */

/* arithmetic of the pair and k-space terms */
#define FMC_PREC_FP64 0 /* everything FP64: parity mode */
#define FMC_PREC_FP32 1 /* FP32 terms; sums and S(k) as FP32 hi/lo pairs */

/* move kinds (the reference's insert / delete / displace flags) */
#define FMC_MOVE_INSERT 1
#define FMC_MOVE_DELETE 2
#define FMC_MOVE_DISPLACE 3  /* "move displace": translation + rotation */
#define FMC_MOVE_TRANSLATE 4 /* "move translate" */
#define FMC_MOVE_ROTATE 5    /* "move rotate" */
#define FMC_MOVE_JUMP 6      /* "move jump" (mc_jump, gcmc.f:1937-2039) */
#define FMC_MOVE_SWAP 7      /* "move swap" (mc_swap, gcmc.f:2269-2452) */

#define FMC_MAX_MOLTYPES 8
#define FMC_MAX_GUEST_TYPES 4
#define FMC_MAX_SITES 8

typedef struct fmc_system fmc_system;
typedef struct fmc_plain fmc_plain;
typedef struct fmc_batch fmc_batch;

/* Copy the calling thread's last error message into buf (NUL-terminated).
 * Returns the message length. */
int fmc_last_error(char *buf, int len);

/* Library version string, e.g. "fastmc_gb300 1.0 sm_103a". */
const char *fmc_version(void);

/* Device allocations (cudaMalloc) and frees (cudaFree) the library has made
 * since it was loaded, over all handles and threads.  A diagnostic with no
 * counterpart in the reference. */
int fmc_alloc_count(int64_t *allocs, int64_t *frees);

/* FP32 FMA throughput of the current device (TFLOP/s, 2 flops per FMA,
 * best of a few launches of an FMA loop on every SM): the denominator of the
 * chain kernel's flop roofline.  A measurement helper with no counterpart in
 * the reference. */
int fmc_measure_fp32_peak(double *tflops);

/* ------------------------------------------------------------- set-up --
 * Replaces: initscan (utility_pack.f:207-508), readfield
 * (readinputs.f:11-307), define_van_der_waals + forgen (vdw_terms.f:1-380),
 * readconfig (readinputs.f:309-513), readcontrol (readinputs.f:515-944),
 * fugacity (utility_pack.f:1206-1310), move-frequency normalisation
 * (gcmc.f:341-386), erfcgen (ewald.f:1-30), lrcorrect (vdw_terms.f:468-684)
 * and excluding_ewald_charges (gcmc.f:2662-2761). */
int fmc_system_load(const char *dir, fmc_system **out);
int fmc_system_free(fmc_system *sys);

typedef struct {
  int imcon;
  int maxmls;       /* molecule types */
  int ntpguest;     /* guest types */
  int ntpatm;       /* unique atom types */
  int n_framework;  /* framework atoms */
  int kmax[3];
  int newld;        /* k-vectors in the half space */
  int mxegrd;       /* table points */
  int guest_mol[FMC_MAX_GUEST_TYPES];    /* locguest */
  int guest_nsites[FMC_MAX_GUEST_TYPES];
  int guest_insert[FMC_MAX_GUEST_TYPES]; /* "create molecules" */
  double alpha, rcut, volm, engunit, temperature, sumchg, drewd;
  double cell[9];
  double fugacity[FMC_MAX_GUEST_TYPES]; /* Pa */
  double ewald3en[FMC_MAX_GUEST_TYPES]; /* per guest type, internal units */
  int mcsteps, eqsteps, nwindsteps;
  double overlap;   /* overlap distance (A) of the trial-position test */
} fmc_system_info;

int fmc_system_get_info(const fmc_system *sys, fmc_system_info *info);

/* The same system from a host that has done the reference's start-up itself
 * (gcmc.f:203-590) and holds its module arrays: the Fortran host's drop-in
 * for fmc_system_load, so the library does not read the input files again.
 * Each field names the reference variable it carries.  Arrays are 0-based
 * copies of the 1-based Fortran ones (element i-1 holds x(i)); 2-D arrays
 * are column-major, as Fortran stores them.  The library enumerates the
 * k-vectors itself from cell, kmax and alpha (ewald.f:151-315) and refuses
 * the system (FMC_ERR_INPUT) when their count differs from the host's newld;
 * everything else, the tables included, is taken as given.  Guests are
 * created on the device (create molecules), so guest molecule types carry
 * nummols 0.  Replaces the host's hand-over of its start-up state; the
 * reference has no such call because its energy routines read the module
 * arrays directly (utility_pack.f:1-204, ewald_module.f, vdw_module.f). */
typedef struct {
  int imcon;               /* imcon: 1 cubic, 2 orthorhombic, 3 parallelepiped */
  double cell[9];          /* cell(1..9) */
  double engunit;          /* engunit (418.4 for UNITS kcal) */
  double temp;             /* temp (K) */
  double rcut;             /* rcut (A) */
  double alpha;            /* alpha, the Ewald convergence parameter (1/A) */
  int kmax[3];             /* kmax1, kmax2, kmax3 */
  int newld;               /* the host's number of k-vectors */
  double epsq;             /* epsq, relative dielectric constant */
  double overlap;          /* overlap distance (A), before the host squares it */
  double surftol;          /* surftol */
  int eqsteps, nwindsteps, minchk, laccsample; /* main-loop control */
  int ntpatm;              /* unique atom types */
  int mxegrd;              /* table points */
  double drewd;            /* erc grid spacing (A) */
  double dlrpot;           /* vvv grid spacing (A) */
  const double *erc;       /* erc(1..mxegrd), erfcgen's table */
  int ntpvdw;              /* van der Waals table rows */
  const double *vvv;       /* vvv(1..mxegrd, 1..ntpvdw), forgen's tables */
  const int *ltpvdw;       /* ltpvdw(1..ntpvdw): 1 = 12-6, 2 = lj */
  const double *prmvdw;    /* prmvdw(1..ntpvdw, 1..2) after define_van_der_waals */
  const int *lstvdw;       /* lstvdw(1..ntpatm*(ntpatm+1)/2): table row per type pair */
  const double *steadd;    /* steadd(1..ntpatm*(ntpatm+1)/2): lrcorrect's tail terms */
  int maxmls;              /* molecule types */
  const int *numatoms;     /* sites per molecule, per molecule type */
  const int *nummols;      /* molecules per type (framework copies; 0 for guests) */
  const int *is_guest;     /* 1 for the &guest molecule types */
  const int *ltype;        /* site atom types 1..ntpatm, type after type */
  const double *charge;    /* site charges, same layout */
  const double *mass;      /* site masses, same layout */
  const int *frozen;       /* site freeze flags, same layout */
  const double *fw_xyz;    /* framework coordinates x,y,z per atom (molxxx/yyy/zzz) */
  int ntpguest;            /* guest types (the &guest types in order) */
  const double *guest_tmpl;/* guestx/y/z: each guest type's centred template */
  const double *fugacity;  /* gstfuga(1..ntpguest), Pa */
  const double *delr;      /* initial displacement size per guest type (A) */
  const double *disp_ratio, *tran_ratio, *rota_ratio; /* acceptance targets */
  const float *move_freq;  /* 8 cumulative REAL*4 thresholds per guest type, in
                              the order mcinsf mcdelf mcdisf mcjmpf mcswpf mctraf
                              mcrotf mcswif (as gcmc.f:341-386 leaves them) */
  const int *create;       /* guest_insert per guest type, or NULL */
} fmc_system_desc;

int fmc_upload_system(const fmc_system_desc *desc, fmc_system **out);

/* Override the fugacity (Pa) of guest type iguest (1-based) before creating
 * chains; used to build isotherms from one set of files. */
int fmc_system_set_fugacity(fmc_system *sys, int iguest, double pascal);

/* --------------------------------------------------- per-move drop-in --
 * One trial-move evaluation per call.  Results in internal units where the
 * reference keeps internal units and kcal/mol (FIELD unit) for estep/delE,
 * as mc_moves.f does. */
typedef struct {
  double estep;     /* energy change, FIELD unit (what energy_eval gets) */
  double ewld1;     /* reciprocal part (ewld1eng), internal units */
  double ewld2;     /* real-space erfc part, internal units */
  double vdw;       /* van der Waals part, internal units */
  double delrc;     /* long-range correction, internal units */
  double delE[FMC_MAX_MOLTYPES]; /* delE(1..maxmls) in delE[0..maxmls-1] */
  int overlap;      /* loverlap */
  int surface;      /* lnewsurf / linitsurf of the evaluated position */
  int surface_old;  /* displacement: linitsurf of the old position */
  int status;       /* device status word (0 = clean) */
  double newxyz[3 * FMC_MAX_SITES]; /* trial site coordinates x,y,z */
} fmc_move_result;

/* Create the device mirror of `sys` (framework, tables, k-vectors) with
 * room for `guest_capacity` molecules per guest type. */
int fmc_plain_create(const fmc_system *sys, int precision, int guest_capacity,
                     fmc_plain **out);
int fmc_plain_destroy(fmc_plain *h);

/* Full reciprocal sum from the current coordinates (ewald.f:354-661) and
 * the electrostatic energy single_point prints (gcmc.f:2659, 585-586):
 * out[0] = ecoul / engunit, out[1] = ewald1 sum (internal), out[2] = sic,
 * out[3] = qfix.  Resets the device S(k) to the recomputed values. */
int fmc_full_ewald(fmc_plain *h, double *out4);

/* The same recomputation, result and S(k) reset as fmc_full_ewald, made
 * without allocating any device memory.  It has no counterpart in the
 * reference (whose ewald1 runs on the host); it is for hosts that cannot let
 * a library allocate in the middle of a run: fmc_full_ewald stages the
 * guests in device buffers it allocates and frees on every call, and a
 * device allocation or free can wait for all work on the device or fail
 * once a host has handed the device's memory to its own allocator.
 *   - Scratch is a fixed 64 KiB array in the library's static device memory
 *     (one partial sum per 8 k-vectors): systems with more than 65528
 *     k-vectors (newld) are refused with FMC_ERR_ARG before anything runs.
 *   - The first call on a device looks up that array's device address
 *     (cudaGetSymbolAddress, with the engine's device current), which may
 *     load the library's kernels on that device; make that first call
 *     before any stream capture on the device.
 *   - Every engine on a device shares the array.  Calls through this entry
 *     point are serialised by a lock held until their kernels finish;
 *     anything else that ran these kernels on the same array at the same
 *     time would race with them.
 *   - The looked-up address is kept for the life of the process.  A
 *     cudaDeviceReset of that device makes it stale: after one, do not call
 *     this entry point on that device again in the same process.
 * Call with the device the engine was created on current (FMC_ERR_ARG
 * otherwise, before anything runs). */
int fmc_full_ewald_noalloc(fmc_plain *h, double *out4);

/* insertion (mc_moves.f:150-276) of guest type iguest at site coordinates
 * xyz (natms triples x,y,z). */
int fmc_insertion(fmc_plain *h, int iguest, const double *xyz,
                  fmc_move_result *res);
/* deletion (mc_moves.f:375-484) of molecule `choice` (1-based). */
int fmc_deletion(fmc_plain *h, int iguest, int choice, fmc_move_result *res);
/* displace_guest (gcmc.f:2816-2901): shift a,b,c then quaternion q1..q4
 * about the new centre of mass; abcq = {a,b,c,q1,q2,q3,q4}. */
int fmc_displace(fmc_plain *h, int iguest, int choice, const double *abcq,
                 fmc_move_result *res);
/* guest_energy (mc_moves.f:277-374) of existing molecule `choice`
 * (lexisting = 1) without a move. */
int fmc_guest_energy(fmc_plain *h, int iguest, int choice,
                     fmc_move_result *res);

/* energy_eval (utility_pack.f:3637-3693) on the device for the last
 * evaluated move, then accept_move / reject_move (mc_moves.f:485-673):
 * commits S(k), coordinates and counters on the device when accepted.
 * `rande` is the host's uniform draw; for a displacement with estep < 0
 * the move is accepted without it (gcmc.f:1879-1886).  Writes the
 * decision to *accepted. */
int fmc_metropolis_commit(fmc_plain *h, double rande, int *accepted);

/* accept_move or reject_move (mc_moves.f:485-673) on the device for the
 * last evaluated move, with the host's own decision (accepted 1 or 0): for
 * a host that keeps calling its energy_eval.  Queued without waiting, like
 * fmc_metropolis_commit; an overlapping trial position is never committed. */
int fmc_commit(fmc_plain *h, int accepted);

/* mc_swap (gcmc.f:2269-2452) in two calls, the host drawing as the
 * reference does.  fmc_swap: molecule `choice` (1-based) of guest type
 * iguest is deleted and committed, a molecule of jguest is built from its
 * template at the deleted molecule's centre of mass, rotated by the
 * quaternion q4 about it, inserted and (unless it overlaps) committed; the
 * result carries both energy changes and the reference's two tests
 * (volume in cubic angstroms, as written there).  The host then decides as
 * gcmc.f:2371-2411 does: if not overlap, rande = duni(); if rande < testi,
 * rande = duni(); accepted if that rande < testj.  fmc_swap_finish(h,
 * accepted) keeps the swap or restores the device state saved before it
 * (an overlapping swap is finished with accepted = 0).  Until then every
 * other move entry point of the engine refuses with FMC_ERR_STATE.  The
 * pair replaces the deletion / accept_move / insertion / accept_move /
 * reject_move sequence of the reference's mc_swap. */
typedef struct {
  double estepi;   /* energy change of the deletion (-estep of deletion) */
  double estepj;   /* energy change of the insertion */
  double testi;    /* first acceptance test (0 when overlap) */
  double testj;    /* second acceptance test (0 when overlap) */
  int overlap;     /* the inserted molecule overlaps */
  int pad;
  double newxyz[3 * FMC_MAX_SITES]; /* inserted site coordinates */
} fmc_swap_result;
int fmc_swap(fmc_plain *h, int iguest, int choice, int jguest, const double *q4,
             fmc_swap_result *res);
int fmc_swap_finish(fmc_plain *h, int accepted);

/* Read back the device state: guest coordinates of guest type iguest
 * (3 * nsites * nummols doubles in molecule order) and the structure
 * factor S(k) per molecule type, [k][moltype][re,im] with moltype
 * 0..maxmls-1 and maxmls = total (2 * (maxmls+1) * newld doubles). */
int fmc_plain_get_nummols(const fmc_plain *h, int iguest, int *n);
int fmc_plain_get_coords(const fmc_plain *h, int iguest, double *xyz, int cap);
int fmc_plain_get_sk(const fmc_plain *h, double *sk, int cap);
/* Guest energies energy(mol), FIELD unit, mol = 1..maxmls. */
int fmc_plain_get_energy(const fmc_plain *h, double *energy, int cap);

/* ------------------------------------------------ device-resident chains */
typedef struct {
  int system;           /* index into the systems array */
  double pressure_pa;   /* fugacity of guest type 1 (< 0: keep the file's) */
  int64_t seed;         /* MZT seed hook (see fmc_batch_create) */
  int create_molecules; /* < 0: use the CONTROL value */
} fmc_chain_spec;

/* Per-chain counters and averages, guest type 1. */
typedef struct {
  int64_t moves;           /* trial moves done */
  int64_t evals;           /* completed energy evaluations (no overlap exit) */
  int64_t overlap_exits;   /* positions rejected by the overlap test */
  int64_t attempts[8];     /* insert, delete, displace, translate, rotate, jump,
                              swap, switch (an acting one) */
  int64_t accepts[8];
  int nummols;
  int status;              /* device status word */
  double energy;           /* energy(guest mol), FIELD unit */
  double avg_n, avg_e, avg_en, avg_n2, avg_e2, avg_nf, qst, cv;
  int64_t prodcount;
  int64_t windows;
  int64_t device_ns;       /* device time of this chain's launches so far */
  double guest_avg_n[FMC_MAX_GUEST_TYPES]; /* <N> of each guest type */
  double guest_se_n[FMC_MAX_GUEST_TYPES];  /* its "standard error" as the
                              reference prints it: the weighted standard
                              deviation of the window averages */
  /* SM clock cycles of the move loop per phase (0 proposal, 1 overlap test,
   * 2 neighbour segments, 3 pair terms, 4 power tables, 5 k-space, 6 block
   * reduction, 7 cluster exchange, 8 epilogue, 9 decision, 10 commit,
   * 11 statistics); zero unless the library was built with
   * FMC_PHASE_TIMERS */
  int64_t phase_cycles[16];
} fmc_chain_stats;

/* One entry of the optional per-move log (parity tests). */
typedef struct {
  int move;      /* FMC_MOVE_* */
  int iguest;
  int choice;
  int overlap;
  int accepted;
  int nmols_after;
  double estep;
  double rande;  /* -1 when not drawn */
  double newxyz[9];
} fmc_move_log;

/* Create `nchains` chains over `nsys` systems.  The seed hook: seed s maps
 * to the clock values the reference would read (milliseconds s % 1000,
 * seconds (s / 1000) % 60, utility_pack.f:2796-2802) and the first draw
 * (gcmc.f:389) is consumed.  "create molecules" pre-loading
 * (mc_moves.f:84-149) runs on the device here.
 * guest_capacity bounds the molecules per chain. */
int fmc_batch_create(const fmc_system *const *systems, int nsys,
                     const fmc_chain_spec *chains, int nchains, int precision,
                     int guest_capacity, fmc_batch **out);
int fmc_batch_destroy(fmc_batch *b);

/* Enable a per-move log of `cap` entries per chain (0 disables). */
int fmc_batch_set_log(fmc_batch *b, int cap);

/* Run `nmoves` main-loop iterations (gcmc.f:704-1164) on every chain.  The
 * cycle is captured once as a CUDA graph and replayed.  If stats != NULL
 * the per-chain statistics are copied to it (nchains entries). */
int fmc_batch_run(fmc_batch *b, int nmoves, fmc_chain_stats *stats);

/* Same, with a host control block: per-chain fugacity (Pa) uploaded
 * before the cycle (nullable), statistics downloaded after it. */
int fmc_batch_run_cycle(fmc_batch *b, int nmoves, const double *host_fugacity,
                        fmc_chain_stats *host_stats);

int fmc_batch_get_stats(fmc_batch *b, fmc_chain_stats *stats);
int fmc_batch_get_log(fmc_batch *b, int chain, fmc_move_log *log, int cap,
                      int *n);
int fmc_batch_get_coords(fmc_batch *b, int chain, double *xyz, int cap, int *n);
/* The same for guest type iguest (1-based); fmc_batch_get_coords is type 1. */
int fmc_batch_get_coords_type(fmc_batch *b, int chain, int iguest, double *xyz, int cap, int *n);
int fmc_batch_get_sk(fmc_batch *b, int chain, double *sk, int cap);

/* Checkpoint / restart of every chain's device state: state records
 * (generator, counters, step sizes, energies, averages), guest coordinates,
 * molecule order and the running S(k), for an exact resume.  The reference
 * writes REVIVE / REVCON files (utility_pack.f:2299-2405) with coordinates
 * and averages only; this file also holds S(k) and the generator.  Load
 * into a batch created from the same systems, chain count, capacity and
 * precision (checked). */
int fmc_batch_save(fmc_batch *b, const char *path);
int fmc_batch_load(fmc_batch *b, const char *path);
/* fmc_batch_load reads and checks the whole file (array sizes, guest counts
 * against the capacity, molecule-order and free-list entries, generator
 * positions, system indices) before any of it reaches the device; a
 * rejected file (FMC_ERR_INPUT) leaves the batch unchanged. */

/* The reference's restart files for one chain (revive,
 * utility_pack.f:2299-2344), written into the existing directory dir:
 * REVIVE, Fortran unformatted sequential records as gfortran writes them
 * (the production flag, nummols of every molecule type, chainstats(1 ..
 * 16 ntpguest + 1) -- the production count and the open window's sums --,
 * the atom count, each molecule type's x, y and z site coordinates, and
 * energy(1 .. ntpguest)); and REVCON, the configuration in CONFIG's layout
 * (guests first, then the framework, as condense orders them).  A
 * reference run restarts from REVIVE with revread (gcmc.f:447-474). */
int fmc_batch_write_revive(fmc_batch *b, int chain, const char *dir);

/* Restart one chain from dir/REVIVE, as the reference does after revread
 * (gcmc.f:447-474) and its start-up: the guest molecules of the file are
 * inserted where they are (no overlap test) and the energies, S(k),
 * counts and charges follow from them; the open window's sums come from
 * the file; the production flag, counters, step sizes, windows and
 * probability grids start again; the chain keeps its generator and
 * pressure.  The framework in the file must be this system's, and the
 * counts must fit the batch's capacity (FMC_ERR_INPUT / FMC_ERR_CAPACITY;
 * nothing is changed then). */
int fmc_batch_read_revive(fmc_batch *b, int chain, const char *dir);

/* The same state copy kept in device memory: fmc_batch_snapshot copies
 * every chain's state, fmc_batch_restore puts that copy back (any number
 * of times), so that cycles can be replayed from one state -- e.g. timed
 * cycles that all start from the same loadings.  No counterpart in the
 * reference. */
int fmc_batch_snapshot(fmc_batch *b);
int fmc_batch_restore(fmc_batch *b);

/* Widom test-particle insertions of guest type iguest (1-based) against
 * chain `chain`'s current state, which they do not change (widom_grid,
 * gcmc.f:2454-2548): trial t is grid point t / nstep (fractions i/ngrid[0],
 * j/ngrid[1], k/ngrid[2], i = 1..ngrid[0] ..., as the reference loops) with
 * a random orientation (random_rot with angle 2 pi about the template
 * origin).  The orientations come from a counter-based hash of (seed,
 * trial), not from the chain's sequential generator, so that all trials run
 * in parallel.  henry = sum over non-overlapping trials of
 * exp(-estep / (kboltz T)) divided by all trials (gcmc.f:2537-2545);
 * counts = {non-overlapping, all}.  Per-trial estep (kcal/mol, 0 for an
 * overlap), overlap flags and site coordinates are optional outputs. */
int fmc_widom_grid(fmc_batch *b, int chain, int iguest, const int *ngrid, int nstep,
                   int64_t seed, double *henry, int64_t *counts, double *estep_out,
                   int *overlap_out, double *xyz_out);
/* The same test insertions at given site coordinates (npos x natms x 3). */
int fmc_widom_positions(fmc_batch *b, int chain, int iguest, int npos, const double *xyz,
                        double *estep_out, int *overlap_out);

/* Probability grids (storeprob, utility_pack.f:621-687; CONTROL
 * "probability" blocks, "grid spacing", "grid factor"): after every
 * production move each guest molecule's centre of mass or listed sites,
 * folded into the unit cell, are spread over 2x2x2 voxels (equitable_bin,
 * utility_pack.f:2407-2519).  ngrid = voxels along a, b, c of the unit
 * cell; nsub = grids of the chain's system (0: none requested).
 * fmc_batch_prob_grid copies grid `sub` (0-based) of one chain: ngrid[0] *
 * ngrid[1] * ngrid[2] doubles, a outer, b middle, c inner, unnormalised
 * (writeprob divides by the voxel volume and prodcount). */
int fmc_batch_prob_info(fmc_batch *b, int chain, int *ngrid, int *nsub);
int fmc_batch_prob_grid(fmc_batch *b, int chain, int sub, double *out, int64_t n);


/* Adjoint of the guest-framework interaction energy (no counterpart in the
 * reference).  For a snapshot of nmol guest molecules (one guest type; site
 * coordinates xyz, nmol x natoms x 3 doubles in DEVICE memory, A):
 *   E = real-space erfc Coulomb + 12-6 Lennard-Jones between guest sites
 *       and framework atoms within the cutoff, + the guest-framework cross
 *       term of the reciprocal Ewald sum (the system's k-vectors), kcal/mol;
 * with per framework atom type t the parameters (eps_t, sigma_t, lambda_t):
 * LJ mixed by Lorentz-Berthelot with the guest sites' self-pair values, and
 * lambda_t a scale of the type-t charges.  fmc_adjoint_eval returns E,
 * dE/dxyz (device, same layout) and dE/dparams (host, ntype x 3).  Exact
 * erfc and analytic LJ (the trial-move path interpolates tables), FP64,
 * orthorhombic cells.  fmc_adjoint_info: number of framework types, guest
 * sites, and the FIELD's parameters (ntype x 3, lambda = 1). */
typedef struct fmc_adjoint fmc_adjoint;
int fmc_adjoint_create(const fmc_system *sys, fmc_adjoint **out);
int fmc_adjoint_info(const fmc_adjoint *a, int *ntype, int *nsite, double *base);
int fmc_adjoint_eval(fmc_adjoint *a, int nmol, const double *xyz, const double *params,
                     double *energy, double *gxyz, double *gparams);
int fmc_adjoint_destroy(fmc_adjoint *a);

/* The energy the chains sample, for a batch of frozen snapshots, and its
 * adjoint.  Per snapshot q (nmol[q] molecules of the system's guest type;
 * xyz: device pointer to every snapshot's site coordinates one after the
 * other, FP64): E_q = the guests' real-space erfc Coulomb and Lennard-Jones
 * terms from the reference's tables (erc, vvv, 3-point interpolation,
 * ewald.f:703-715, vdw_terms.f:441-453) against the framework and the
 * other molecules, the reciprocal sum of the guests with the framework and
 * with each other (each molecule's own |s_m|^2 included: it turns with the
 * molecule), and the guest-framework Lennard-Jones tail (lrcorrect,
 * vdw_terms.f:470-645), in kcal/mol: the sampled energy up to terms that
 * depend only on the molecule count (the framework's own energy also on
 * lambda, equally in every snapshot).  xyz and gxyz may be null when every
 * snapshot is empty.  params (host, ntype x 3): framework type t's (eps_t,
 * sigma_t, lambda_t); its pairs' parameters move from the FIELD's values
 * as Lorentz-Berthelot mixing does and lambda_t scales its charges.
 * Out: energy[q] (host), gxyz (device, float, 3 per site: dE/dxyz),
 * gparams[q][t][3] (host).  precision: FMC_PREC_FP64 (pair terms and
 * phases in FP64) or FMC_PREC_FP32 (in FP32, sums in FP64).  Orthorhombic
 * cells, one guest type.  The handle keeps its device buffers between
 * calls (grown to the largest batch): one call at a time per handle.  No
 * counterpart in the reference. */
int fmc_adjoint_eval_batch(fmc_adjoint *a, int nsnap, const int *nmol, const double *xyz,
                           const double *params, int precision, double *energy, float *gxyz,
                           double *gparams);

/* Thread-block clusters: the chains of system i run on clusters of
 * csize[i] CTAs (1..8; default 1).  Each CTA of a cluster takes a share of
 * the chain's framework atoms, guests and k-vectors; results do not depend
 * on the cluster size beyond the order of the final sums.  nsys must be the
 * batch's number of systems.  No counterpart in the reference (its chains
 * are MPI ranks of one core each). */
int fmc_batch_set_cluster(fmc_batch *b, const int *csize, int nsys);
/* The same per chain (nchains sizes): heavily loaded chains of a system can
 * get more CTAs than its light ones.  fmc_batch_get_cluster then reports
 * each system's largest size.  Size 0 pauses a chain (it is not run until
 * it gets a size again); at least one chain must stay active. */
int fmc_batch_set_chain_cluster(fmc_batch *b, const int *csize, int nchains);
int fmc_batch_get_chain_cluster(const fmc_batch *b, int *csize, int nchains);
/* Speculative proposals in FP32 batches of one guest type with resident
 * guests: up to kmax (2..8) moves are drawn ahead, their overlap tests run
 * as one block-wide pass, the leading overlap exits are completed together
 * and the draws of the proposals after the first one that passes are
 * undone, so the chains' moves, draws and decisions are those of the
 * sequential loop.  0 or 1: off (the default).  No reference counterpart:
 * the reference runs one move at a time (gcmc.f:704-1164). */
int fmc_batch_set_speculation(fmc_batch *b, int kmax);

int fmc_batch_get_cluster(const fmc_batch *b, int *csize, int nsys);

/* Autotuner: picks the cluster size of every system by timing trial cycles
 * of `nmoves` moves from a copy of the chains' state: starting from one CTA
 * per chain, it doubles the cluster of every system whose slowest chain is
 * within 20% of the cycle time, while the cycle gets more than 3% faster.
 * It sets the choice and restores the chains' state, so the chains continue
 * exactly as if it had not run.  csize_out (nullable) receives the choice. */
int fmc_batch_autotune(fmc_batch *b, int nmoves, int *csize_out, int nsys);

/* Timing of the last fmc_batch_run: device milliseconds of the persistent
 * kernel (CUDA events on its stream) and the completed evaluations. */
int fmc_batch_last_timing(const fmc_batch *b, double *kernel_ms,
                          int64_t *evals, int64_t *moves);

/* Bytes one fmc_batch_run_cycle call copies host -> device (the fugacity
 * array, when given) and device -> host (every chain's state record, from
 * which the statistics are filled).  A measurement helper; no counterpart
 * in the reference. */
int fmc_batch_cycle_bytes(const fmc_batch *b, int64_t *h2d, int64_t *d2h);

#ifdef __cplusplus
}
#endif
#endif

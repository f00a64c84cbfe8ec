/*
 * fmc_oracle.h -- C API of the CPU FP64 oracle for the FastMC GCMC
 * trial-move energy path.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is a plain C++ restatement of the
 * reference Fortran (ewald.f, vdw_terms.f, mc_moves.f, utility_pack.f,
 * gcmc.f, readinputs.f, parse_module.f) that the CUDA path is tested
 * against, and the timed CPU baseline.  Nothing in fastmc_gb300/ links,
 * loads or calls it.
 *
 * Parity pin: the initial electrostatic energy of the reference's own
 * CALF-20 test system (test/CONFIG + test/FIELD, cutoff 12.5, ewald
 * precision 1d-6) must equal -11190.606165 kcal/mol (run_test.py:39).
 *
 * All routines are single threaded and FP64, except the MZT random number
 * generator, which is REAL*4 as in the reference (utility_pack.f:2768).
 */
#ifndef FMC_ORACLE_H
#define FMC_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_sim orc_sim;

/* Last error message of the calling thread (empty string if none). */
const char *orc_last_error(void);

/* Read FIELD, CONFIG and CONTROL from directory `dir` and perform the
 * reference start-up sequence (gcmc.f:203-590): initscan, readfield,
 * readconfig, readcontrol, fugacity, move-frequency normalisation,
 * condense, erfcgen, single_point.  Returns NULL on error. */
orc_sim *orc_create(const char *dir);
void orc_destroy(orc_sim *s);

/* Energies printed by the reference after single_point (gcmc.f:575-590),
 * in the FIELD energy unit: out[0]=van der Waals (vdwsum+elrc)/engunit,
 * out[1]=electrostatic ecoul/engunit, out[2]=DL_POLY energy/engunit,
 * out[3]=ewald1 reciprocal sum (internal units), out[4]=alpha,
 * out[5]=kmax1, out[6]=kmax2, out[7]=kmax3, out[8]=newld (k-vector count),
 * out[9]=volume, out[10]=engunit, out[11]=sumchg, out[12]=overlap
 * distance (A). */
void orc_setup_energies(const orc_sim *s, double *out);

/* Seed the MZT generator deterministically.  The reference seeds from the
 * wall clock (utility_pack.f:2796-2802) with values(8)=milliseconds and
 * values(7)=seconds; the hook maps seed -> ms = seed % 1000,
 * sec = (seed / 1000) % 60 and applies the same formulas.  The first
 * duni() call of the reference (gcmc.f:389, returns 0) is performed here. */
void orc_seed(orc_sim *s, long long seed);

/* Integer sizes / scalars. */
int orc_ntpguest(const orc_sim *s);
int orc_maxmls(const orc_sim *s);
int orc_nummols(const orc_sim *s, int mol);        /* 1-based molecule type */
int orc_numatoms(const orc_sim *s, int mol);
int orc_locguest(const orc_sim *s, int iguest);    /* 1-based guest index */
int orc_newld(const orc_sim *s);
double orc_energy(const orc_sim *s, int mol);      /* energy(mol), kcal/mol */

/* Copy coordinates of molecule type `mol` (molxxx layout: nummols*numatoms
 * rows, x,y,z per row) into out (3*n doubles, row-major x,y,z). Returns n. */
int orc_get_coords(const orc_sim *s, int mol, double *out, int cap);

/* Structure factor ckcsum/ckssum(i, k) for i = 1..maxmls+1 (maxmls+1 is
 * the total), k = 1..newld.  out receives 2*(maxmls+1)*newld doubles laid
 * out [k][i][re,im].  Returns newld. */
int orc_get_sk(const orc_sim *s, double *out, int cap);

/* Per-move results (the values the reference computes for one move). */
typedef struct {
  int move;          /* 1 insert, 2 delete, 3 displace, 4 translate, 5 rotate,
                        6 jump, 7 swap, 8 switch, 0 a switch that returned
                        without acting */
  int iguest;        /* 1-based guest type */
  int choice;        /* 1-based molecule picked (delete/displace), 0 for insert */
  int overlap;       /* loverlap of the trial position */
  int accepted;
  int nmols_after;   /* nummols(mol) after the move */
  double estep;      /* energy change in kcal/mol as passed to energy_eval */
  double rande;      /* uniform draw used by energy_eval, -1 if not drawn */
  double dele_other; /* sum of delE(i) for i != mol (kcal/mol) */
  double newxyz[9];  /* trial site coordinates (first 3 sites), x,y,z each */
} orc_move_log;

/* Run `nsteps` iterations of the GCMC main loop (gcmc.f:704-1164 for the
 * insert / delete / displace / translate / rotate moves).  If log != NULL
 * it receives one record per step (cap >= nsteps).  Returns steps run, or
 * -1 on error. */
int orc_run(orc_sim *s, int nsteps, orc_move_log *log, int cap);

/* gstfuga(iguest) in Pa after set-up (fugacity, utility_pack.f:1206-1310). */
double orc_fugacity(const orc_sim *s, int iguest);

/* One swap (mc_swap, gcmc.f:2269-2452) with its draws given: molecule
 * `choice` of iguest replaced by a molecule of jguest at its centre of mass,
 * rotated by q[0..3]; rande[0..1] are the two Metropolis numbers.
 * out: [0] estepi, [1] estepj, [2] loverlap, [3] accepted.  0 or -1. */
int orc_swap(orc_sim *s, int iguest, int choice, int jguest, const double *q,
             const double *rande, double *out);

/* "create molecules" pre-loading (mc_moves.f:84-149), as gcmc.f:664-690
 * does for each guest with guest_insert > 0.  Returns the number of trials
 * or -1 on error. */
int orc_create_molecules(orc_sim *s, int iguest, int nguests);

/* insert_guests' framework pre-test (on by default): trial positions that
 * certainly overlap a framework atom skip insertion(), which would reject
 * them without leaving any state behind; the created molecules and the
 * generator's sequence are the same with it on or off. */
void orc_set_prefilter(orc_sim *s, int on);

/* The set-up arrays of fmc_upload_system's descriptor (fmc_system_desc),
 * by field name, as doubles: the oracle playing the Fortran host that has
 * done the reference's start-up.  Returns the element count (out == NULL:
 * the count only), -count when cap is too small, -1 for an unknown name. */
int orc_get_array(const orc_sim *s, const char *name, double *out, int cap);

/* Keep a copy of the whole simulation state (coordinates, S(k), energies,
 * counters, generator) and put it back: replays of one state. 0 or -1. */
int orc_save_state(orc_sim *s);
int orc_restore_state(orc_sim *s);

/* Stand-alone energy routines for parity of the C-ABI entry points.
 * Coordinates are site-major x,y,z triples (natms sites).  The state of
 * the simulation is not changed, except the scratch arrays the reference
 * itself overwrites (ckcsnew/ckssnew, ewald1en, ...).
 * out: [0]=estep (kcal/mol), [1]=ewld1eng, [2]=ewld2sum, [3]=vdwsum,
 *      [4]=delrc, [5]=overlap flag, [6]=surface flag, [7..7+maxmls)=delE. */
int orc_insertion_energy(orc_sim *s, int iguest, const double *xyz, double *out);
int orc_deletion_energy(orc_sim *s, int iguest, int choice, double *out);
/* displace_guest with explicit shift (a,b,c) and quaternion q1..q4.  S(k)
 * is restored afterwards, as the reject path of mc_displace does. */
int orc_displace_energy(orc_sim *s, int iguest, int choice, const double *abcq,
                        double *out);

/* Commit a move with explicit inputs, exactly as mc_insert / mc_delete /
 * mc_displace would after the given decision.  kind: 1 insert (xyz),
 * 2 delete (choice), 3 displace (choice, abcq). accepted: 0/1. */
int orc_apply_move(orc_sim *s, int kind, int iguest, int choice,
                   const double *xyz_or_abcq, int accepted);

/* Statistics (gcmc.f:1050-1128, 1168-1258) for guest iguest:
 * out[0..7] = <N>,<E>,<EN>,<N2>,<E2>,<NF>,Qst,Cv ; out[8] = production
 * steps; out[9] = number of windows.  Acceptance counters:
 * out[10..13] = ins_count, accept_ins, del_count, accept_del,
 * out[14..17] = disp_count, accept_disp, rota_count, accept_rota,
 * out[18..19] = tran_count, accept_tran,
 * out[20..22] = delrdisp, rotangle, rota_rotangle,
 * out[23..24] = jump_count, accept_jump,
 * out[25..28] = swap_count, accept_swap, switch_count, accept_switch,
 * out[29] = the "standard error" of <N> (gcmc.f:1218-1241)
 * (out holds 30 doubles). */
void orc_stats(const orc_sim *s, int iguest, double *out);
/* probability grids (storeprob): out4 = ngrida, ngridb, ngridc, number of
 * subgrids (0 when none is requested); grid `sub` (1-based) as gridsize
 * doubles, bin order a outer, b middle, c inner */
int orc_prob_info(const orc_sim *s, int *out4);
int orc_prob_grid(const orc_sim *s, int sub, double *out, int n);
/* storeenprob of given site coordinates (natms x 3) and energy, as
 * widom_grid calls it for a test insertion */
int orc_store_energy(orc_sim *s, int iguest, const double *xyz, double energy);
long long orc_prodcount(const orc_sim *s);

/* MZT generator alone (for RNG parity tests): seed like orc_seed on a
 * private generator and draw n numbers (the initialising call excluded). */
void orc_duni_sequence(long long seed, int n, double *out);

/* Tables as uploaded by the host: erc(1..mxegrd) and vvv(1..mxegrd, k).
 * Returns mxegrd. */
int orc_get_erc(const orc_sim *s, double *out, int cap);
int orc_get_vvv(const orc_sim *s, int k, double *out, int cap);

#ifdef __cplusplus
}
#endif
#endif

// fmc_oracle.cpp -- CPU FP64 oracle for the FastMC GCMC trial-move energy path.
//
// TEST INFRASTRUCTURE ONLY: what the CUDA path is tested against, and the
// timed CPU baseline.  The product library never links or loads this file.
//
// This is a plain C++ restatement of the reference Fortran.  Every routine
// names the reference routine and file:line it follows.  Arrays keep the
// reference's 1-based indices so each loop can be compared line by line.
// Parity is pinned by the reference's own known answer: the initial
// electrostatic energy of test/CONFIG + test/FIELD is -11190.606165
// (run_test.py:39, printed at gcmc.f:585-586).
//
// Build: -O3 -ffp-contract=off (no FMA contraction, so x86-64 and aarch64
// give identical results; the REAL*4 generator depends on it).

#include "fmc_oracle.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

// ---------------------------------------------------------------- constants
// utility_pack.f:81-147 and parse_module.f:9
constexpr int LENREC = 150;
constexpr double PI = 3.141592653589793;
constexpr double SQRPI = 1.7724538509055159;
constexpr double R4PIE0 = 138935.4835;
constexpr double KBOLTZ = 1.9872041e-3;
constexpr double BOLTZ = 1.3806503e-23;
constexpr double RGAS = 8.314472 / 4184.0;
constexpr double MINANGLE = PI / 18.0;
constexpr double DELRMIN = 0.1;

thread_local std::string g_err;

struct Fail : std::runtime_error {
  using std::runtime_error::runtime_error;
};

[[noreturn]] void fail(const std::string &m) { throw Fail(m); }

// ------------------------------------------------------------ parse_module
// A record is LENREC characters, blank padded (parse_module.f:9-11).
struct Rec {
  char c[LENREC];
  char &operator()(int i) { return c[i - 1]; }  // 1-based like the Fortran
  char operator()(int i) const { return c[i - 1]; }
};

// getrec (parse_module.f:15-79): read one line, keep 150 columns.
bool getrec(FILE *f, Rec &r) {
  char buf[4096];
  if (!std::fgets(buf, sizeof buf, f)) return false;
  size_t n = std::strlen(buf);
  while (n && (buf[n - 1] == '\n' || buf[n - 1] == '\r')) --n;
  for (int i = 0; i < LENREC; ++i) r.c[i] = (size_t)i < n ? buf[i] : ' ';
  return true;
}

// lowcase (parse_module.f:291-369)
void lowcase(Rec &r, int length) {
  int m = length < 255 ? length : 255;
  if (m > LENREC) m = LENREC;
  for (int i = 1; i <= m; ++i)
    if (r(i) >= 'A' && r(i) <= 'Z') r(i) = char(r(i) - 'A' + 'a');
}

// strip (parse_module.f:258-289): drop leading blanks.
void strip(Rec &r, int imax) {
  for (int i = 1; i <= imax; ++i) {
    if (r(1) == ' ') {
      for (int j = 1; j <= imax - 1; ++j) r(j) = r(j + 1);
      r(imax) = ' ';
    }
  }
}

// findstring (parse_module.f:393-427)
bool findstring(const char *seek, const Rec &r) {
  int n = (int)std::strlen(seek);
  for (int here = 0; here <= LENREC - n; ++here) {
    bool ok = true;
    for (int i = 1; i <= n; ++i)
      if (seek[i - 1] != r(here + i)) { ok = false; break; }
    if (ok) return true;
  }
  return false;
}

// shift helper shared by intstr/dblstr (parse_module.f:139-144)
void shift_word(char *w, int len, int lst) {
  for (int j = lst; j <= len; ++j) w[j - lst] = w[j - 1];
  for (int j = len - lst + 2; j <= len; ++j) w[j - 1] = ' ';
}

// intstr (parse_module.f:81-146): first integer in the string; consumes it.
int intstr_raw(char *w, int len, int &lst) {
  int isn = 1, val = 0;
  char ksn = '+';
  bool count = false, fin = false;
  lst = 0;
  while (lst < len && !fin) {
    ++lst;
    bool flag = false;
    char ch = w[lst - 1];
    if (ch >= '0' && ch <= '9') {
      val = 10 * val + (ch - '0');
      count = true;
      flag = true;
    }
    if (count && !flag) fin = true;
    if (flag && ksn == '-') isn = -1;
    ksn = ch;
  }
  val *= isn;
  shift_word(w, len, lst);
  return val;
}
int intstr(Rec &r) {
  int lst;
  return intstr_raw(r.c, LENREC, lst);
}

// 10.d0**iexp with an integer exponent (Fortran real**integer).
double pow10i(int e) {
  double p = 1.0;
  int a = e < 0 ? -e : e;
  for (int i = 0; i < a; ++i) p *= 10.0;
  return e < 0 ? 1.0 / p : p;
}

// dblstr (parse_module.f:148-256): first real in the string; consumes it.
// Digits accumulate as val = ten*val + one*j with one divided by ten after
// the decimal point, exactly as the reference does.
double dblstr_raw(char *w, int len) {
  int lst = 0, iexp = 0, idum = 0;
  double sn = 1.0, ten = 10.0, one = 1.0, val = 0.0;
  char ksn = '+';
  bool start = false, ldot = false, fin = false;
  while (lst < len && !fin) {
    ++lst;
    bool flag = false;
    char ch = w[lst - 1];
    if (ch >= '0' && ch <= '9') {
      double t1 = ten * val;
      double t2 = one * double(ch - '0');
      val = t1 + t2;
      flag = true;
      start = true;
    }
    if (ch == '.') {
      flag = true;
      ten = 1.0;
      ldot = true;
      start = true;
    }
    if (flag && ksn == '-') sn = -1.0;
    if (ldot) one = one / 10.0;
    ksn = ch;
    if (ksn == 'D') ksn = 'd';
    if (ksn == 'E') ksn = 'e';
    if (start) {
      if (ksn == 'd' || ksn == 'e') {
        std::vector<char> work(len > lst ? len - lst : 1, ' ');
        for (int i = 1; i <= len - lst; ++i) work[i - 1] = w[i + lst - 1];
        iexp = intstr_raw(work.data(), len - lst, idum);
        fin = true;
      }
      if (!flag) fin = true;
    }
  }
  val = sn * val * pow10i(iexp);
  lst += idum;
  shift_word(w, len, lst);
  return val;
}
double dblstr(Rec &r) { return dblstr_raw(r.c, LENREC); }

// getword (parse_module.f:547-602): next blank-delimited word, len1 chars.
std::string getword(Rec &r, int len1) {
  std::string seq(len1, ' ');
  int i = 0, k = 0;
  bool fin = false;
  while (!fin && i < LENREC) {
    ++i;
    if (r(1) == ' ') {
      if (k > 0) fin = true;
    } else {
      ++k;
      seq[k - 1] = r(1);
      if (k == len1) fin = true;
    }
    for (int j = 1; j <= LENREC - 1; ++j) r(j) = r(j + 1);
    r(LENREC) = ' ';
  }
  std::string w = seq;
  w.resize(8, ' ');
  return w;
}

// loc2 (utility_pack.f:2859-2872), loc8 (3005-3018)
inline int loc2(int i, int j) {
  int a = i > j ? i : j, b = i > j ? j : i;
  return (a * (a - 1)) / 2 + b;
}

// Fortran NINT: round half away from zero.
inline double fnint(double x) { return std::round(x); }

// --------------------------------------------------------------- geometry
// invert (utility_pack.f:1962-2004)
void invert(const double *a, double *b, double &d) {
  b[0] = a[4] * a[8] - a[5] * a[7];
  b[1] = a[2] * a[7] - a[1] * a[8];
  b[2] = a[1] * a[5] - a[2] * a[4];
  b[3] = a[5] * a[6] - a[3] * a[8];
  b[4] = a[0] * a[8] - a[2] * a[6];
  b[5] = a[2] * a[3] - a[0] * a[5];
  b[6] = a[3] * a[7] - a[4] * a[6];
  b[7] = a[1] * a[6] - a[0] * a[7];
  b[8] = a[0] * a[4] - a[1] * a[3];
  d = a[0] * b[0] + a[3] * b[1] + a[6] * b[2];
  double r = 0.0;
  if (std::fabs(d) > 0.0) r = 1.0 / d;
  for (int i = 0; i < 9; ++i) b[i] = r * b[i];
}

// dcell (utility_pack.f:1904-1960)
void dcell(const double *a, double *b) {
  b[0] = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  b[1] = std::sqrt(a[3] * a[3] + a[4] * a[4] + a[5] * a[5]);
  b[2] = std::sqrt(a[6] * a[6] + a[7] * a[7] + a[8] * a[8]);
  b[3] = (a[0] * a[3] + a[1] * a[4] + a[2] * a[5]) / (b[0] * b[1]);
  b[4] = (a[0] * a[6] + a[1] * a[7] + a[2] * a[8]) / (b[0] * b[2]);
  b[5] = (a[3] * a[6] + a[4] * a[7] + a[5] * a[8]) / (b[1] * b[2]);
  double axb1 = a[1] * a[5] - a[2] * a[4];
  double axb2 = a[2] * a[3] - a[0] * a[5];
  double axb3 = a[0] * a[4] - a[1] * a[3];
  double bxc1 = a[4] * a[8] - a[5] * a[7];
  double bxc2 = a[5] * a[6] - a[3] * a[8];
  double bxc3 = a[3] * a[7] - a[4] * a[6];
  double cxa1 = a[7] * a[2] - a[1] * a[8];
  double cxa2 = a[0] * a[8] - a[2] * a[6];
  double cxa3 = a[1] * a[6] - a[0] * a[7];
  b[9] = std::fabs(a[0] * bxc1 + a[1] * bxc2 + a[2] * bxc3);
  b[6] = b[9] / std::sqrt(bxc1 * bxc1 + bxc2 * bxc2 + bxc3 * bxc3);
  b[7] = b[9] / std::sqrt(cxa1 * cxa1 + cxa2 * cxa2 + cxa3 * cxa3);
  b[8] = b[9] / std::sqrt(axb1 * axb1 + axb2 * axb2 + axb3 * axb3);
}

// images (utility_pack.f:1697-1902), imcon 1, 2 and 3.
void images(int imcon, int n, const double *cell, double *x, double *y,
            double *z) {
  if (imcon == 1) {
    double aaa = 1.0 / cell[0];
    for (int i = 0; i < n; ++i) {
      x[i] = x[i] - cell[0] * fnint(aaa * x[i]);
      y[i] = y[i] - cell[0] * fnint(aaa * y[i]);
      z[i] = z[i] - cell[0] * fnint(aaa * z[i]);
    }
  } else if (imcon == 2) {
    double aaa = 1.0 / cell[0], bbb = 1.0 / cell[4], ccc = 1.0 / cell[8];
    for (int i = 0; i < n; ++i) {
      x[i] = x[i] - cell[0] * fnint(aaa * x[i]);
      y[i] = y[i] - cell[4] * fnint(bbb * y[i]);
      z[i] = z[i] - cell[8] * fnint(ccc * z[i]);
    }
  } else if (imcon == 3) {
    double rc[9], det;
    invert(cell, rc, det);
    for (int i = 0; i < n; ++i) {
      double ssx = rc[0] * x[i] + rc[3] * y[i] + rc[6] * z[i];
      double ssy = rc[1] * x[i] + rc[4] * y[i] + rc[7] * z[i];
      double ssz = rc[2] * x[i] + rc[5] * y[i] + rc[8] * z[i];
      double xss = ssx - fnint(ssx), yss = ssy - fnint(ssy),
             zss = ssz - fnint(ssz);
      x[i] = cell[0] * xss + cell[3] * yss + cell[6] * zss;
      y[i] = cell[1] * xss + cell[4] * yss + cell[7] * zss;
      z[i] = cell[2] * xss + cell[5] * yss + cell[8] * zss;
    }
  } else if (imcon != 0) {
    fail("oracle: imcon " + std::to_string(imcon) + " not supported");
  }
}

// ------------------------------------------------------------ MZT generator
// duni (utility_pack.f:2768-2857): Marsaglia-Zaman-Tsang universal
// generator with REAL*4 state.
struct Duni {
  float u[97];
  float c = 0, cd = 0, cm = 0;
  int ir = 97, jr = 33;
  bool fresh = true;

  void init_from_clock(int ms, int sec) {
    int i = (ms * 3) % 177 + 1;
    int j = (sec * 23) % 177 + 1;
    int k = (ms * 5) % 177 + 1;
    int l = (sec * 3) % 168;
    ir = 97;
    jr = 33;
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
      u[ii] = s;
    }
    c = 362436.0f / 16777216.0f;
    cd = 7654321.0f / 16777216.0f;
    cm = 16777213.0f / 16777216.0f;
    fresh = false;
  }
  double next() {
    if (fresh) fail("oracle: duni used before seeding");
    float uni = u[ir - 1] - u[jr - 1];
    if (uni < 0.0f) uni = uni + 1.0f;
    u[ir - 1] = uni;
    ir = ir - 1;
    if (ir == 0) ir = 97;
    jr = jr - 1;
    if (jr == 0) jr = 97;
    c = c - cd;
    if (c < 0.0f) c = c + cm;
    uni = uni - c;
    if (uni < 0.0f) uni = uni + 1.0f;
    return double(uni);
  }
};

void seed_to_clock(long long seed, int &ms, int &sec) {
  long long s = seed < 0 ? -seed : seed;
  ms = int(s % 1000);
  sec = int((s / 1000) % 60);
}

// ------------------------------------------------------------------ model
struct MolType {
  std::string name;
  bool guest = false;
  int nummols = 0, natoms = 0;
  std::vector<std::string> atmname;  // 1-based
  std::vector<double> wght, chg;
  std::vector<int> frz, ltp;
  std::vector<double> mx, my, mz;  // molxxx(mol, :) 1-based
};

constexpr int kMaxProbSites = 64;

struct Sim {
  // ------------------------------------------------------------ inputs
  int imcon = 0, levcfg = 0;
  double cell[9] = {0}, rcell[9] = {0}, celprp[10] = {0};
  double volm = 0, statvolm = 0;
  double engunit = 1.0, sumchg = 0.0;
  int maxmls = 0, ntpmls = 0, ntpguest = 0, ntpfram = 0, ntpatm = 0;
  int mxatyp = 0, ntpvdw = 0, maxvdw = 0, totatm = 0;
  std::vector<MolType> mol;              // 1-based molecule types
  std::vector<int> locguest, locfram;    // 1-based
  std::vector<std::string> unqatm;       // 1-based
  std::vector<std::vector<double>> guestx, guesty, guestz;  // [iguest][site]
  std::vector<double> molmass;
  // van der Waals (vdw_module.f)
  int mxegrd = 0;
  std::vector<int> ltpvdw, lstvdw;
  std::vector<std::vector<double>> prmvdw;  // [ivdw][1..5]
  std::vector<std::vector<double>> vvv;     // [ivdw][1..mxegrd]
  std::vector<double> steadd;
  double dlrpot = 0;
  double elrc = 0;
  std::vector<double> elrc_mol, delrc_mol, delrc_mol0;
  std::vector<int> numtyp, numfrz;                   // [atype]
  std::vector<std::vector<int>> numtyp_mol, numfrz_mol;        // [mol][atype]
  std::vector<std::vector<int>> numtyp_gstmol, numfrz_gstmol;  // [iguest][atype]
  std::vector<double> vdwen, vdwentmp;
  // control
  double temp = 0, rcut = 0, rvdw = 0, initdelr = 0, eps = 0, alpha = 0;
  int kmax1 = 0, kmax2 = 0, kmax3 = 0, keyfce = 0;
  int mcsteps = 1, eqsteps = 0, nwind = 1, nwindsteps = 1, nnumg = 1;
  int nhis = 0;
  bool lspe = false, laccsample = false;
  // probability grids (gcmc.f:258-306, storeprob utility_pack.f:621-687)
  double griddim = 0.1;
  int gridfactor[3] = {1, 1, 1};
  bool lprob = false;
  int ntprob = 0;
  std::vector<int> nprob, lprobeng;                 // [iguest]
  std::vector<int> nprobsites;                      // [1..ntprob]
  std::vector<std::vector<int>> lprobsites;         // [1..ntprob][1..]
  int ngrida = 0, ngridb = 0, ngridc = 0, gridsize = 0;
  double ucell[9] = {0}, rucell[9] = {0};
  std::vector<double> grid;                         // [(sub - 1) * gridsize + bin - 1]
  double overlap = 1.5, surftol = 0.0;
  std::vector<double> gstpress, gstfuga, gstmolfract, delr;
  bool lfuga = false;
  std::vector<float> mcinsf, mcdelf, mcdisf, mcjmpf, mcswpf, mctraf, mcrotf,
      mcswif, mcmvnorm;
  std::vector<double> disp_ratio, tran_ratio, rota_ratio;
  std::vector<int> guest_insert;
  double total_pressure = -1.0;
  double beta = 0, epsq = 1.0, drewd = 0;
  // ewald (ewald_module.f)
  int mxebuf = 0, newld = 0;
  std::vector<double> ckcsum, ckssum, ckcsnew, ckssnew, ckcsorig, ckssorig;
  std::vector<double> erc, fer;
  std::vector<double> ewald1en, ewald2en, ewald3en, engsic, engsicorig,
      chgsum_mol, ewald1entmp, ewald2entmp;
  // condensed arrays (utility_pack.f)
  std::vector<double> xxx, yyy, zzz, atmcharge, atmweight;
  std::vector<int> ltype, moltype, lfreezesite;
  // per-move scratch
  std::vector<double> newx, newy, newz;
  std::vector<int> ind, ilist, moldf;
  std::vector<double> xdf, ydf, zdf, rsqdf;
  std::vector<int> gstlentry;
  std::vector<std::vector<int>> gstlist;
  std::vector<double> delE, energy, surfacemols;
  // move control and counters
  std::vector<double> delrdisp, tran_delr;
  double rotangle = PI / 3.0, rota_rotangle = PI / 3.0;
  std::vector<long long> ins_count, accept_ins, del_count, accept_del,
      disp_count, accept_disp, tran_count, accept_tran, rota_count,
      accept_rota, jump_count, accept_jump, swap_count, accept_swap, switch_count,
      accept_switch;
  // mc_swap's saved long-range corrections (gcmc.f:2312-2313); mc_switch
  // restores them on rejection although it never sets them itself
  double origelrc = 0.0;
  std::vector<double> origelrc_mol;
  // statistics
  bool production = false;
  bool last_accepted = false;  // the main loop's `accepted` (not reset per move)
  int cur_iguest = 1;          // the main loop's iguest (the move's guest type)
  long long gcmccount = 0, prodcount = 0, rollcount = 0, cycle_step = 0;
  int minchk = 1;
  std::vector<double> chainstats;
  std::vector<std::vector<double>> avgwindow;  // [window][1..]
  Duni rng;
  bool prefilter_inserts = true;  // insert_guests' framework pre-test (fw_overlap_certain)
  // results of set-up
  double spe_vdw = 0, spe_ecoul = 0, spe_dlpeng = 0, ewald1sum = 0;

  int mxcmls() const { return maxmls * (maxmls - 1) / 2 + maxmls; }
  double &ckc(std::vector<double> &v, int i, int k) {
    return v[(size_t)(i - 1) + (size_t)(k - 1) * (maxmls + 1)];
  }

  // ---------------------------------------------------------- input readers
  void read_all(const std::string &dir);
  void initscan(const std::string &dir);
  void readfield(const std::string &dir);
  void define_van_der_waals(FILE *f);
  void forgen();
  void readconfig(const std::string &dir);
  void readcontrol(const std::string &dir);
  void fugacity();
  void normalise_moves();
  // ------------------------------------------------------------ energies
  void condense();
  void erfcgen();
  void lrcorrect();
  void gstlrcorrect(int iguest, double &delrc, bool lexisting);
  void ewald1(double &engcpe, double &engsicold);
  void ewald1_guest(double &engcpe, int natms, int iguest, double &chgtmp,
                    double &engsictmp, bool lexisting);
  void ewald2(double chg, int natm, double &engcpe, int molt);
  void ewald3(double chg, int molt, int natms, const std::vector<int> &jlist,
              double &engcpe);
  void srfrce(int sittyp, int ik, int molt, double &engsrp);
  void excluding_ewald_charges(double &ewald3sum);
  void single_point();
  void surface_check(int iatm, int j, int molt, bool &loverlap,
                     bool &latmsurf);
  // -------------------------------------------------------------- moves
  void insertion(int iguest, double &delrc, double &estep, double &chgtmp,
                 double &engsictmp, bool &loverlap, bool &lnewsurf,
                 double *parts);
  void guest_energy(int iguest, double &vdwsum, double &ewld2sum,
                    double &ewld1eng, bool &lsurf, double &chgtmp,
                    double &engsictmp, bool &loverlap, double &estep,
                    bool lexisting);
  void deletion(int iguest, int choice, double &delrc, double &estep,
                bool &linitsurf, double &engsictmp, double &chgtmp,
                double *parts);
  void displace_guest(int iguest, int imol, double a, double b, double c,
                      double q1, double q2, double q3, double q4,
                      bool &linitsurf, bool &lnewsurf, bool &loverlap,
                      double &estep);
  void accept_move(int iguest, bool insert, bool del, bool disp, bool lsurf,
                   double delrc, int &choice, double engsictmp, double chgtmp);
  void reject_move(int iguest, bool insert, bool del, bool disp);
  bool energy_eval(double eng, double rande, int iguest, bool displace,
                   bool insert, bool del);
  void get_guest(int iguest, int choice, int &molt, int &natms, int &nmols);
  void random_ins(int iguest);
  void random_disp(double ddelr, double &a, double &b, double &c);
  void random_rot(double rotang, double &q1, double &q2, double &q3,
                  double &q4);
  void cartesian(double fa, double fb, double fc, double &x, double &y,
                 double &z) const;
  void com(int natms, int molt, double &cx, double &cy, double &cz) const;
  void rotation(int natms, double cx, double cy, double cz, double q1,
                double q2, double q3, double q4);
  void translate(int natms, int molt, double a, double b, double c);
  // driver
  void mc_insert(int iguest, orc_move_log *lg);
  void mc_delete(int iguest, orc_move_log *lg);
  void mc_displace(int iguest, bool tran, bool rota, orc_move_log *lg);
  void mc_jump(int iguest, orc_move_log *lg);
  // the swap itself, with its molecule, partner type and quaternion given;
  // rande[0..1] are the Metropolis numbers, or null to draw them
  void swap_move(int iguest, int ichoice, int jguest, const double *q,
                 const double *rande, double *out, orc_move_log *lg);
  void mc_swap(int iguest, orc_move_log *lg);
  void mc_switch(int iguest, orc_move_log *lg);
  void step(orc_move_log *lg);
  int insert_guests(int iguest, int nguests);
  // Pre-loading only: the framework atoms on a cell grid, so that
  // insert_guests can skip trial positions that certainly overlap a
  // framework atom without the full list build of insertion().
  struct FwGrid {
    bool built = false;
    int nc[3] = {0, 0, 0};
    double csz[3] = {0, 0, 0};
    std::vector<int> start;            // [cell] -> first atom, cells z fastest
    std::vector<double> x, y, z;       // atoms sorted by cell
  } fwgrid;
  bool fw_overlap_certain(int natms);
  void production_stats(bool accepted);
  void storeenprob(int iguest, double energy);
  void setup_grid();
  void equitable_bin(double fa, double fb, double fc, int sub, double val);
  void storeprob();
};

std::string path_join(const std::string &d, const char *f) {
  if (d.empty()) return f;
  return d + "/" + f;
}

FILE *open_or_fail(const std::string &p) {
  FILE *f = std::fopen(p.c_str(), "r");
  if (!f) fail("oracle: cannot open " + p);
  return f;
}

// initscan (utility_pack.f:207-508): sizes, cell, cutoff, Ewald parameters.
void Sim::initscan(const std::string &dir) {
  Rec r;
  mxatyp = 0;
  keyfce = 0;
  std::vector<std::string> chr;
  FILE *f = open_or_fail(path_join(dir, "FIELD"));
  if (!getrec(f, r)) fail("oracle: empty FIELD");
  bool loop = true;
  while (loop) {
    if (!getrec(f, r)) fail("oracle: FIELD ended before close");
    lowcase(r, LENREC);
    strip(r, LENREC);
    if (r(1) == '#' || r(1) == ' ') {
    } else if (findstring("molecu", r)) {
      maxmls = intstr(r);
      int nummls = 0;
      for (int n = 1; n <= maxmls; ++n) {
        bool loop2 = true;
        while (loop2) {
          if (!getrec(f, r)) fail("oracle: FIELD truncated");
          lowcase(r, LENREC);
          strip(r, LENREC);
          if (r(1) == '#' || r(1) == ' ') {
          } else if (findstring("nummol", r)) {
            nummls = intstr(r);
          } else if (findstring("atoms", r)) {
            int numsit = intstr(r);
            int ksite = 0;
            for (int isite = 1; isite <= numsit; ++isite) {
              if (ksite < numsit) {
                if (!getrec(f, r)) fail("oracle: FIELD truncated");
                std::string name = getword(r, 8);
                dblstr(r);
                dblstr(r);
                int nrept = intstr(r);
                intstr(r);
                intstr(r);
                if (nrept == 0) nrept = 1;
                ksite += nrept;
                bool check = true;
                for (auto &c : chr)
                  if (c == name) check = false;
                if (check) chr.push_back(name);
              }
            }
          } else if (findstring("finish", r)) {
            loop2 = false;
          }
        }
      }
    } else if (findstring("vdw", r)) {
      ntpvdw = intstr(r);
    } else if (findstring("close", r)) {
      loop = false;
    }
  }
  std::fclose(f);
  mxatyp = (int)chr.size();
  // CONFIG header: imcon and cell (utility_pack.f:327-348)
  f = open_or_fail(path_join(dir, "CONFIG"));
  getrec(f, r);
  getrec(f, r);
  imcon = intstr(r);
  imcon = intstr(r);
  for (int row = 0; row < 3; ++row) {
    if (!getrec(f, r)) fail("oracle: CONFIG truncated");
    cell[3 * row + 0] = dblstr(r);
    cell[3 * row + 1] = dblstr(r);
    cell[3 * row + 2] = dblstr(r);
  }
  std::fclose(f);
  dcell(cell, celprp);
  // CONTROL (utility_pack.f:349-440)
  f = open_or_fail(path_join(dir, "CONTROL"));
  bool lcut = false, ldelr = false, lwind = false, lrvdw = false,
       lewald = false;
  bool loop3 = true;
  while (loop3) {
    if (!getrec(f, r)) fail("oracle: CONTROL ended before finish");
    lowcase(r, LENREC);
    strip(r, LENREC);
    if (r(1) == '#' || r(1) == ' ') {
    } else if (findstring("cut", r)) {
      rcut = dblstr(r);
      lcut = true;
    } else if (findstring("&guest", r)) {
      bool loop4 = true;
      while (loop4) {
        if (!getrec(f, r)) fail("oracle: CONTROL guest block truncated");
        lowcase(r, LENREC);
        strip(r, LENREC);
        if (r(1) == '#' || r(1) == ' ') {
        } else if (findstring("probability", r)) {  // utility_pack.f:360-380
          int qprob = intstr(r);
          lprob = true;
          ntprob += qprob;
          int iprob = 0;
          while (iprob < qprob) {
            if (!getrec(f, r)) fail("oracle: CONTROL truncated");
            strip(r, LENREC);
            if (r(1) == '#' || r(1) == ' ') {
            } else if (r(1) == 'e') {
              ++ntprob;
              ++iprob;
            } else {
              ++iprob;
            }
          }
        } else if (findstring("&end", r)) {
          loop4 = false;
        }
      }
    } else if (findstring("henry", r)) {
    } else if (findstring("grid", r)) {  // utility_pack.f:436-443
      if (findstring("spa", r)) {
        griddim = dblstr(r);
      } else if (findstring("fac", r)) {
        gridfactor[0] = intstr(r);
        gridfactor[1] = intstr(r);
        gridfactor[2] = intstr(r);
      }
    } else if (findstring("delr", r)) {
      initdelr = dblstr(r);
      ldelr = true;
    } else if (findstring("averaging window", r)) {
      nwind = intstr(r);
      lwind = true;
    } else if (findstring("steps", r)) {
      mcsteps = intstr(r);
    } else if (findstring("finish", r)) {
      loop3 = false;
    } else if (findstring("ewald", r)) {
      lewald = true;
      keyfce = 2;
      if (findstring("precision", r)) {
        eps = dblstr(r);
        if (!lcut) fail("oracle: ewald precision before cutoff (error 433)");
        eps = std::fmin(std::fabs(eps), 0.5);
        double tol = std::sqrt(std::fabs(std::log(eps * rcut)));
        alpha = std::sqrt(std::fabs(std::log(eps * rcut * tol))) / rcut;
        double t = 2.0 * tol * alpha;
        double tol1 = std::sqrt(-std::log(eps * rcut * (t * t)));
        double fac = 1.0;
        if (imcon == 4 || imcon == 5 || imcon == 7)
          fac = std::pow(2.0, 1.0 / 3.0);
        kmax1 = (int)fnint(0.25 + fac * celprp[0] * alpha * tol1 / PI);
        kmax2 = (int)fnint(0.25 + fac * celprp[1] * alpha * tol1 / PI);
        kmax3 = (int)fnint(0.25 + fac * celprp[2] * alpha * tol1 / PI);
      } else {
        alpha = dblstr(r);
        kmax1 = intstr(r);
        kmax2 = intstr(r);
        kmax3 = intstr(r);
      }
    } else if (findstring("rvdw", r)) {
      rvdw = dblstr(r);
      lrvdw = true;
    }
  }
  std::fclose(f);
  if (!ldelr) fail("oracle: delr missing in CONTROL (error 433)");
  int cfactor = std::abs(mcsteps);
  if (!lwind) nwind = cfactor > 1000 ? 5 : 1;
  nwindsteps = (int)std::ceil(double(cfactor) / double(nwind));
  if (nwindsteps < 1) nwindsteps = 1;
  nwind = (int)std::floor(double(cfactor) / double(nwindsteps));
  double width = std::fmin(celprp[6], std::fmin(celprp[7], celprp[8])) / 2.0;
  if (rcut > width) fail("oracle: cutoff exceeds half cell width (error 95)");
  if (imcon == 4 || imcon == 5 || imcon == 7)
    volm = 0.5 * celprp[9];
  else if (imcon == 0)
    volm = 0.0;
  else
    volm = celprp[9];
  if (!lrvdw && rcut > 0.0) rvdw = rcut;
  if (!lewald) fail("oracle: no ewald directive (error 2311)");
  maxvdw = std::max(ntpvdw, (mxatyp * (mxatyp + 1)) / 2);
  // alloc_config_arrays / alloc_vdw_arrays (utility_pack.f:928-1204,
  // vdw_module.f:32-79)
  mxegrd = std::max(1000, int(rvdw / 0.01 + 0.5) + 4);
}

// readfield (readinputs.f:11-307)
void Sim::readfield(const std::string &dir) {
  Rec r;
  FILE *f = open_or_fail(path_join(dir, "FIELD"));
  mol.assign(maxmls + 1, MolType());
  locguest.assign(maxmls + 1, 0);
  locfram.assign(maxmls + 1, 0);
  unqatm.assign(1, "");
  guestx.assign(maxmls + 1, {});
  guesty.assign(maxmls + 1, {});
  guestz.assign(maxmls + 1, {});
  molmass.assign(maxmls + 1, 0.0);
  ltpvdw.assign(maxvdw + 2, -1);
  lstvdw.assign(maxvdw + 2, 0);
  prmvdw.assign(maxvdw + 2, std::vector<double>(6, 0.0));
  vvv.assign(maxvdw + 2, std::vector<double>(mxegrd + 3, 0.0));
  ntpatm = 0;
  ntpguest = ntpfram = 0;
  totatm = 0;
  engunit = 1.0;
  getrec(f, r);
  bool loop = true;
  while (loop) {
    if (!getrec(f, r)) fail("oracle: FIELD ended before close");
    lowcase(r, LENREC);
    strip(r, LENREC);
    if (findstring("units", r)) {
      bool blank = true;
      for (int i = 6; i <= LENREC; ++i)
        if (r(i) != ' ') blank = false;
      if (blank) {
      } else if (findstring("ev", r)) {
        engunit = 9648.530821;
      } else if (findstring("kcal", r)) {
        engunit = 418.4;
      } else if (findstring("kj", r)) {
        engunit = 1.0e2;
      } else if (findstring("k", r)) {
        engunit = BOLTZ;
      }
    } else if (findstring("vdw", r)) {
      define_van_der_waals(f);
    } else if (findstring("molecu", r)) {
      ntpmls = intstr(r);
      sumchg = 0.0;
      for (int n = 1; n <= ntpmls; ++n) {
        MolType &m = mol[n];
        double mass = 0.0;
        bool lguest = false;
        if (!getrec(f, r)) fail("oracle: FIELD truncated");
        lowcase(r, LENREC);
        if (findstring("&guest", r)) {
          lguest = true;
          ++ntpguest;
          locguest[ntpguest] = n;
          m.guest = true;
        } else {
          ++ntpfram;
          locfram[ntpfram] = n;
        }
        m.name = std::string(r.c, 40);
        bool loop2 = true;
        while (loop2) {
          if (!getrec(f, r)) fail("oracle: FIELD truncated");
          lowcase(r, LENREC);
          strip(r, LENREC);
          if (findstring("nummol", r)) {
            m.nummols = intstr(r);
          } else if (findstring("atoms", r)) {
            int numsit = intstr(r);
            m.natoms = numsit;
            m.atmname.assign(numsit + 1, "");
            m.wght.assign(numsit + 1, 0.0);
            m.chg.assign(numsit + 1, 0.0);
            m.frz.assign(numsit + 1, 0);
            m.ltp.assign(numsit + 1, 0);
            if (lguest) {
              guestx[ntpguest].assign(numsit + 1, 0.0);
              guesty[ntpguest].assign(numsit + 1, 0.0);
              guestz[ntpguest].assign(numsit + 1, 0.0);
            }
            int ksite = 0;
            for (int isite = 1; isite <= numsit; ++isite) {
              if (ksite >= numsit) continue;
              if (!getrec(f, r)) fail("oracle: FIELD truncated");
              std::string atom1 = getword(r, 8);
              double weight = dblstr(r);
              double charge = dblstr(r);
              int nrept, ifrz;
              if (lguest) {
                nrept = 1;
                guestx[ntpguest][isite] = dblstr(r);
                guesty[ntpguest][isite] = dblstr(r);
                guestz[ntpguest][isite] = dblstr(r);
                ifrz = 0;
              } else {
                nrept = intstr(r);
                ifrz = intstr(r);
              }
              if (nrept == 0) nrept = 1;
              for (int ir = 1; ir <= nrept; ++ir) {
                ++ksite;
                if (ksite > numsit) fail("oracle: FIELD repeat overflow");
                m.atmname[ksite] = atom1;
                m.wght[ksite] = weight;
                m.chg[ksite] = charge;
                m.frz[ksite] = ifrz;
                mass += weight;
              }
              bool atmchk = true;
              for (int js = 1; js <= ntpatm; ++js) {
                if (atom1 == unqatm[js]) {
                  atmchk = false;
                  for (int ir = ksite; ir >= ksite - nrept + 1; --ir)
                    m.ltp[ir] = js;
                }
              }
              if (atmchk) {
                ++ntpatm;
                unqatm.push_back(atom1);
                for (int ir = ksite; ir >= ksite - nrept + 1; --ir)
                  m.ltp[ir] = ntpatm;
              }
            }
          } else if (findstring("finish", r)) {
            loop2 = false;
            if (lguest) {
              // readinputs.f:221-243.  `mass` already holds the site
              // masses from the ATOMS loop; the reference adds them a
              // second time before dividing, so the subtracted centre is
              // sum(m_i r_i) / (2 M).  Kept as is.
              molmass[n] = mass;
              double cx = 0, cy = 0, cz = 0;
              for (int i = 1; i <= m.natoms; ++i) {
                cx += guestx[ntpguest][i] * m.wght[i];
                cy += guesty[ntpguest][i] * m.wght[i];
                cz += guestz[ntpguest][i] * m.wght[i];
                mass += m.wght[i];
              }
              cx /= mass;
              cy /= mass;
              cz /= mass;
              for (int i = 1; i <= m.natoms; ++i) {
                guestx[ntpguest][i] -= cx;
                guesty[ntpguest][i] -= cy;
                guestz[ntpguest][i] -= cz;
              }
            } else {
              molmass[n] = mass * m.nummols;
            }
          }
        }
        totatm += m.natoms * m.nummols;
      }
    } else if (findstring("close", r)) {
      loop = false;
    } else {
      fail("oracle: unrecognised FIELD directive");
    }
  }
  std::fclose(f);
  for (int it = 1; it <= ntpmls; ++it)
    for (int ls = 1; ls <= mol[it].natoms; ++ls)
      sumchg = sumchg + double(mol[it].nummols) * mol[it].chg[ls];
}

// define_van_der_waals (vdw_terms.f:1-179)
void Sim::define_van_der_waals(FILE *f) {
  Rec r;
  for (int i = 1; i <= maxvdw; ++i) {
    lstvdw[i] = 0;
    ltpvdw[i] = -1;
  }
  dlrpot = 0.0;
  for (int it = 1; it <= ntpvdw; ++it) {
    double parpot[6] = {0, 0, 0, 0, 0, 0};
    if (!getrec(f, r)) fail("oracle: VDW block truncated");
    std::string atom1 = getword(r, 8);
    std::string atom2 = getword(r, 8);
    lowcase(r, LENREC - 16);
    std::string kw = getword(r, 4).substr(0, 4);
    int keypot = -1;
    if (kw == "12-6") keypot = 1;
    else if (kw == "lj  ") keypot = 2;
    else if (kw == "nm  ") keypot = 3;
    else if (kw == "buck") keypot = 4;
    else if (kw == "bhm ") keypot = 5;
    else if (kw == "hbnd") keypot = 6;
    else if (kw == "snm " || kw == "hcnm") keypot = 7;
    else if (kw == "mors") keypot = 8;
    else if (kw == "wca ") keypot = 9;
    else if (kw == "tab ") keypot = 0;
    if (keypot != 1 && keypot != 2)
      fail("oracle: only lj and 12-6 van der Waals forms are restated");
    for (int i = 1; i <= 5; ++i) parpot[i] = dblstr(r);
    int k1 = 0, k2 = 0;
    for (int j = 1; j <= ntpatm; ++j) {
      if (atom1 == unqatm[j]) k1 = j;
      if (atom2 == unqatm[j]) k2 = j;
    }
    if (k1 == 0 || k2 == 0) fail("oracle: VDW line names an unknown atom");
    int keyvdw = loc2(k1, k2);
    parpot[1] *= engunit;
    if (keypot == 1) parpot[2] *= engunit;
    lstvdw[keyvdw] = it;
    ltpvdw[it] = keypot;
    for (int i = 1; i <= 5; ++i) prmvdw[it][i] = parpot[i];
  }
  if (ntpvdw > 0) forgen();
  int ntab = (ntpatm * (ntpatm + 1)) / 2;
  if (ntpvdw < ntab) {
    for (int i = 1; i <= ntab; ++i)
      if (lstvdw[i] == 0) lstvdw[i] = ntpvdw + 1;
    for (int i = 1; i <= mxegrd; ++i) vvv[ntpvdw + 1][i] = 0.0;
  }
}

// forgen (vdw_terms.f:181-234; lj and 12-6 forms)
void Sim::forgen() {
  dlrpot = rvdw / double(mxegrd - 4);
  for (int iv = 1; iv <= ntpvdw; ++iv) {
    if (ltpvdw[iv] == 1) {
      double aaa = prmvdw[iv][1], bbb = prmvdw[iv][2];
      for (int i = 1; i <= mxegrd; ++i) {
        double rrr = double(i) * dlrpot;
        double r6 = std::pow(rrr, 6);
        vvv[iv][i] = (aaa / r6 - bbb) / r6;
      }
    } else if (ltpvdw[iv] == 2) {
      double e = prmvdw[iv][1], s = prmvdw[iv][2];
      for (int i = 1; i <= mxegrd; ++i) {
        double rrr = double(i) * dlrpot;
        double sr6 = std::pow(s / rrr, 6);
        vvv[iv][i] = 4.0 * e * sr6 * (sr6 - 1.0);
      }
    }
  }
}

// readconfig (readinputs.f:309-513)
void Sim::readconfig(const std::string &dir) {
  Rec r;
  FILE *f = open_or_fail(path_join(dir, "CONFIG"));
  getrec(f, r);
  getrec(f, r);
  levcfg = intstr(r);
  if (imcon == 0) {
    for (double &c : cell) c = 0.0;
  } else {
    for (int row = 0; row < 3; ++row) {
      if (!getrec(f, r)) fail("oracle: CONFIG truncated");
      cell[3 * row + 0] = dblstr(r);
      cell[3 * row + 1] = dblstr(r);
      cell[3 * row + 2] = dblstr(r);
    }
  }
  char line[4096];
  auto read_line = [&](std::string &out) {
    if (!std::fgets(line, sizeof line, f)) fail("oracle: CONFIG truncated");
    out = line;
    while (!out.empty() && (out.back() == '\n' || out.back() == '\r'))
      out.pop_back();
  };
  // format (3f20.0): three fixed 20-column fields
  auto read3 = [&](double &a, double &b, double &c) {
    std::string s;
    read_line(s);
    s.resize(60, ' ');
    a = std::strtod(s.substr(0, 20).c_str(), nullptr);
    b = std::strtod(s.substr(20, 20).c_str(), nullptr);
    c = std::strtod(s.substr(40, 20).c_str(), nullptr);
  };
  for (int k = 1; k <= maxmls; ++k) {
    MolType &m = mol[k];
    int n = m.nummols * m.natoms;
    m.mx.assign(n + 1, 0.0);
    m.my.assign(n + 1, 0.0);
    m.mz.assign(n + 1, 0.0);
    int indatm = 0;
    for (int l = 1; l <= m.nummols; ++l) {
      for (int a = 1; a <= m.natoms; ++a) {
        ++indatm;
        std::string nm;
        read_line(nm);
        nm.resize(8, ' ');
        Rec rn;
        std::memset(rn.c, ' ', LENREC);
        for (int i = 0; i < 8; ++i) rn.c[i] = nm[i];
        strip(rn, 8);
        std::string atname(rn.c, 8);
        double x, y, z, junk;
        read3(x, y, z);
        if (levcfg >= 1) read3(junk, junk, junk);
        if (levcfg >= 2) read3(junk, junk, junk);
        if (m.atmname[a] != atname)
          fail("oracle: unidentified atom label in CONFIG (error 25)");
        m.mx[indatm] = x;
        m.my[indatm] = y;
        m.mz[indatm] = z;
      }
    }
  }
  std::fclose(f);
  dcell(cell, celprp);
  if (imcon == 4 || imcon == 5 || imcon == 7)
    volm = 0.5 * celprp[9];
  else if (imcon == 0)
    volm = 0.0;
  else
    volm = celprp[9];
  if (imcon > 0) {
    double width = std::fmin(celprp[6], std::fmin(celprp[7], celprp[8])) / 2.0;
    if (rcut > width) fail("oracle: cutoff exceeds half cell width (error 95)");
  }
}

// readcontrol (readinputs.f:515-944): the directives the GCMC path uses.
void Sim::readcontrol(const std::string &dir) {
  Rec r;
  FILE *f = open_or_fail(path_join(dir, "CONTROL"));
  gstpress.assign(ntpguest + 1, -1.0);
  gstmolfract.assign(ntpguest + 1, -1.0);
  total_pressure = -1.0;
  double tmp[8] = {-1, -1, -1, -1, -1, -1, -1, -1};  // ins del dis jum swa swi tra rot
  double tmpdisp = -1, tmptran = -1, tmprota = -1;
  bool ltemp = false, lmcsteps = false, leqsteps = false, lnumg = false;
  int ngst = 0, piprob = 0;
  nprob.assign(ntpguest + 1, 0);
  lprobeng.assign(ntpguest + 1, 0);
  nprobsites.assign(ntprob + 1, 0);
  lprobsites.assign(ntprob + 1, std::vector<int>());
  getrec(f, r);
  bool loop = true;
  while (loop) {
    if (!getrec(f, r)) fail("oracle: CONTROL ended before finish");
    lowcase(r, LENREC);
    strip(r, LENREC);
    if (r(1) == '#' || r(1) == ' ') {
    } else if (findstring("block", r)) {
      fail("oracle: pore blocking is not restated");
    } else if (findstring("henry", r)) {
    } else if (findstring("widom ins", r)) {
      intstr(r);
    } else if (findstring("restart", r)) {
      fail("oracle: restart is not restated");
    } else if (findstring("temp", r)) {
      temp = dblstr(r);
      ltemp = true;
    } else if (findstring("sampling", r)) {
      laccsample = true;
    } else if (findstring("&guest", r)) {
      ++ngst;
      int idg = intstr(r);
      if (idg < 1 || idg > ntpguest) fail("oracle: bad &guest index");
      bool rprob = false;
      bool loop2 = true;
      while (loop2) {
        if (!getrec(f, r)) fail("oracle: CONTROL guest block truncated");
        lowcase(r, LENREC);
        strip(r, LENREC);
        if (r(1) == '#' || r(1) == ' ') {
        } else if (findstring("fract", r)) {
          gstmolfract[idg] = dblstr(r);
        } else if (findstring("create molecules", r)) {
          guest_insert[idg] = intstr(r);
        } else if (findstring("min molecules", r)) {
          intstr(r);
        } else if (findstring("max molecules", r)) {
          intstr(r);
        } else if (findstring("press", r)) {
          gstpress[idg] = dblstr(r) * 1.0e5;
        } else if (findstring("probability", r)) {  // readinputs.f:642-672
          rprob = true;
          bool leng = false;
          int nnprob = intstr(r);
          nprob[idg] = nnprob;
          int cprob = 0;
          while (cprob < nnprob) {
            if (!getrec(f, r)) fail("oracle: CONTROL truncated");
            strip(r, LENREC);
            if (r(1) == '#' || r(1) == ' ') {
            } else if (r(1) == 'e') {
              leng = true;
              ++cprob;
            } else {
              ++piprob;
              ++cprob;
              int ntpsite = intstr(r);
              if ((int)nprobsites.size() <= piprob) {
                nprobsites.resize(piprob + 1, 0);
                lprobsites.resize(piprob + 1);
              }
              nprobsites[piprob] = ntpsite;
              lprobsites[piprob].assign(ntpsite + 1, 0);
              for (int j = 1; j <= ntpsite; ++j) lprobsites[piprob][j] = intstr(r);
            }
          }
          if (leng) {
            lprobeng[idg] = 1;
            nprob[idg] += 1;
          }
        } else if (findstring("move", r)) {
          if (findstring("ins", r)) mcinsf[idg] = (float)dblstr(r);
          else if (findstring("del", r)) mcdelf[idg] = (float)dblstr(r);
          else if (findstring("dis", r)) mcdisf[idg] = (float)dblstr(r);
          else if (findstring("jum", r)) mcjmpf[idg] = (float)dblstr(r);
          else if (findstring("swa", r)) mcswpf[idg] = (float)dblstr(r);
          else if (findstring("swi", r)) mcswif[idg] = (float)dblstr(r);
          else if (findstring("tra", r)) mctraf[idg] = (float)dblstr(r);
          else if (findstring("rot", r)) mcrotf[idg] = (float)dblstr(r);
        } else if (findstring("delr", r)) {
          delr[idg] = dblstr(r);
        } else if (findstring("accep", r)) {
          if (findstring("dis", r)) disp_ratio[idg] = dblstr(r);
          else if (findstring("tra", r)) tran_ratio[idg] = dblstr(r);
        } else if (findstring("&end", r)) {
          loop2 = false;
        }
      }
      if (!rprob) nprob[ngst] = 0;  // readinputs.f:706 (indexed by the block count)
    } else if (findstring("steps", r)) {
      mcsteps = intstr(r);
      lmcsteps = true;
    } else if (findstring("pressure", r) || findstring("total press", r)) {
      total_pressure = dblstr(r) * 1.0e5;
    } else if (findstring("numg", r)) {
      lnumg = true;
      nnumg = intstr(r);
      if (nnumg <= 0) nnumg = 1000;
    } else if (findstring("fuga", r)) {
      lfuga = true;
    } else if (findstring("hist", r)) {
      nhis = intstr(r);
    } else if (findstring("equilibr", r)) {
      eqsteps = intstr(r);
      if (eqsteps != 0) leqsteps = true;
    } else if (findstring("wang-landau", r)) {
      fail("oracle: Wang-Landau is not restated");
    } else if (findstring("uvt", r)) {
    } else if (findstring("single point", r)) {
      lspe = true;
    } else if (findstring("jobcontrol", r)) {
      fail("oracle: jobcontrol is not restated");
    } else if (findstring("cutoff", r)) {
      rcut = dblstr(r);
    } else if (findstring("overlap", r)) {
      overlap = dblstr(r);
    } else if (findstring("surface", r)) {
      surftol = dblstr(r);
    } else if (findstring("delr", r)) {
      dblstr(r);
    } else if (findstring("averaging window", r)) {
    } else if (findstring("max", r)) {
    } else if (findstring("move", r)) {
      if (findstring("ins", r)) tmp[0] = dblstr(r);
      else if (findstring("del", r)) tmp[1] = dblstr(r);
      else if (findstring("dis", r)) tmp[2] = dblstr(r);
      else if (findstring("jum", r)) tmp[3] = dblstr(r);
      else if (findstring("swa", r)) tmp[4] = dblstr(r);
      else if (findstring("swi", r)) tmp[5] = dblstr(r);
      else if (findstring("tra", r)) tmp[6] = dblstr(r);
      else if (findstring("rot", r)) tmp[7] = dblstr(r);
    } else if (findstring("accep", r)) {
      if (findstring("dis", r)) tmpdisp = dblstr(r);
      else if (findstring("tra", r)) tmptran = dblstr(r);
      else if (findstring("rot", r)) tmprota = dblstr(r);
    } else if (findstring("grid", r)) {
    } else if (findstring("finish", r)) {
      loop = false;
    } else if (findstring("ewald", r)) {
    } else {
      fail("oracle: unknown CONTROL directive (error 3)");
    }
  }
  std::fclose(f);
  (void)tmpdisp;
  (void)tmptran;
  (void)tmprota;
  std::vector<float> *mv[8] = {&mcinsf, &mcdelf, &mcdisf, &mcjmpf,
                               &mcswpf, &mcswif, &mctraf, &mcrotf};
  for (int ig = 1; ig <= ngst; ++ig)
    for (int q = 0; q < 8; ++q)
      if ((*mv[q])[ig] < 0.0f) (*mv[q])[ig] = tmp[q] >= 0.0 ? (float)tmp[q] : 0.0f;
  if (!leqsteps) eqsteps = 0;
  if (!lnumg) nnumg = eqsteps > 1000 ? eqsteps / 1000 : 1;
  if (!lmcsteps) {
    mcsteps = 1;
    lspe = true;
  }
  if (ngst != ntpguest) fail("oracle: guest blocks do not match FIELD (error 2312)");
  if (!ltemp) fail("oracle: no temperature (error 380)");
}

// fugacity (utility_pack.f:1206-1310) with fluid_properties / guess_guest
// (utility_pack.f:1311-1424) and calc_fugacity (utility_pack.f:1428-1500).
// REAL*4 literals of the reference are kept as float values; K_fug, which
// the reference allocates without setting (apart from CH4 + C2H6), is zero.
void Sim::fugacity() {
  bool lfract = false, lpress = true;
  double fract_sum = 0, press_sum = 0, no_fract = 0;
  for (int i = 1; i <= ntpguest; ++i) {
    if (gstpress[i] < 0.0) lpress = false;
    else press_sum += gstpress[i];
    if (gstmolfract[i] > 0.0) {
      lfract = true;
      fract_sum += gstmolfract[i];
    } else {
      no_fract += 1.0;
    }
  }
  if (lfract && !lpress) {
    if (total_pressure < 0.0) fail("oracle: error 2314");
    if (ntpguest == 1) {
      gstmolfract[1] = 1.0;
      fract_sum = 1.0;
    }
    if (fract_sum < 1.0)
      for (int i = 1; i <= ntpguest; ++i)
        if (gstmolfract[i] < 0) gstmolfract[i] = (1.0 - fract_sum) / no_fract;
    for (int i = 1; i <= ntpguest; ++i)
      gstpress[i] = total_pressure * gstmolfract[i];
  }
  if (!lpress && !lfract && total_pressure > 0.0) {
    for (int i = 1; i <= ntpguest; ++i) gstpress[i] = total_pressure;
    total_pressure = ntpguest * total_pressure;
    press_sum = total_pressure;
  }
  if (total_pressure > 0.0 && !lfract) {
    if (press_sum != total_pressure) total_pressure = press_sum;
    for (int i = 1; i <= ntpguest; ++i) gstmolfract[i] = gstpress[i] / total_pressure;
  } else if (lpress && !lfract) {
    total_pressure = press_sum;
    for (int i = 1; i <= ntpguest; ++i) gstmolfract[i] = gstpress[i] / total_pressure;
  }
  gstfuga.assign(ntpguest + 1, 0.0);
  // fluid_properties: Acc_factor, T_crit, P_crit by guess_guest's mass bins
  std::vector<double> acc(ntpguest + 1), tcrit(ntpguest + 1), pcrit(ntpguest + 1);
  std::vector<int> iguess(ntpguest + 1, 0);
  bool fuga_on = lfuga;
  for (int j = 1; j <= ntpguest && lfuga; ++j) {
    const MolType &m = mol[locguest[j]];
    double mass = 0.0;
    for (int i = 1; i <= m.natoms; ++i) mass += m.wght[i];
    int g = 0;
    if (mass > 27.0 && mass < 29.0) g = 1;
    else if (mass > 43.0 && mass < 45.0) g = 2;
    else if (mass > 15.5 && mass < 17.0) g = 3;
    else if (mass > 29.0 && mass < 31.0) g = 4;
    else if (mass > 1.0 && mass < 3.0) g = 5;
    iguess[j] = g;
    switch (g) {
      case 1: acc[j] = 0.037f; tcrit[j] = 126.2f; pcrit[j] = 3.398e6f; break;
      case 2: acc[j] = 0.225f; tcrit[j] = 304.12f; pcrit[j] = 7.374e6f; break;
      case 3: acc[j] = 0.011f; tcrit[j] = 190.56f; pcrit[j] = 4.599e6f; break;
      case 4: acc[j] = 0.099f; tcrit[j] = 305.32f; pcrit[j] = 4.872e6f; break;
      case 5: acc[j] = -0.217f; tcrit[j] = 32.98f; pcrit[j] = 1.293e6f; break;
      default: fuga_on = false;
    }
  }
  if (!fuga_on) {
    for (int i = 1; i <= ntpguest; ++i) gstfuga[i] = gstpress[i];
    return;
  }
  std::vector<std::vector<double>> kfug(ntpguest + 1, std::vector<double>(ntpguest + 1, 0.0));
  if (ntpguest == 2 && ((iguess[1] == 3 && iguess[2] == 4) || (iguess[1] == 4 && iguess[2] == 3))) {
    kfug[1][2] = -0.003f;
    kfug[2][1] = kfug[1][2];
  }
  // calc_fugacity for each guest type
  const double R = 8.314f;
  for (int ig = 1; ig <= ntpguest; ++ig) {
    std::vector<double> kappa(ntpguest + 1), alphaT(ntpguest + 1), ag(ntpguest + 1), bg(ntpguest + 1);
    for (int i = 1; i <= ntpguest; ++i) {
      kappa[i] = double(0.37464f) + double(1.54226f) * acc[i] - double(0.26992f) * acc[i] * acc[i];
      double t = 1 + kappa[i] * (1 - std::sqrt(temp / tcrit[i]));
      alphaT[i] = t * t;
      double rt = R * tcrit[i];
      ag[i] = double(0.45724f) * (rt * rt) / pcrit[i] * alphaT[i];
      bg[i] = double(0.0778f) * R * tcrit[i] / pcrit[i];
    }
    double as = 0.0, bs = 0.0;
    if (ntpguest == 1) {
      as = ag[1];
      bs = bg[1];
    } else {
      for (int i = 1; i <= ntpguest; ++i) {
        for (int j = 1; j <= ntpguest; ++j)
          as = as + gstmolfract[i] * gstmolfract[j] * std::sqrt(ag[i] * ag[j]) * (1 - kfug[i][j]);
        bs = bs + gstmolfract[i] * bg[i];
      }
    }
    const double rT = R * temp;
    const double A = as * gstpress[ig] / (rT * rT);
    const double B = bs * gstpress[ig] / R / temp;
    const double alpha = B - 1, beta_f = A - 3 * B * B - 2 * B, gamma = -A * B + B * B + B * B * B;
    double z1 = 1.0, z0;
    int iter = 0;
    do {
      if (++iter > 10000) fail("oracle: Peng-Robinson compressibility did not converge");
      z0 = z1;
      z1 = z0 - (z0 * z0 * z0 + alpha * (z0 * z0) + beta_f * z0 + gamma) /
                    (3 * (z0 * z0) + 2 * alpha * z0 + beta_f);
    } while (!(std::fabs(z1 - z0) < 1.0e-5));
    double sum_za = 0.0;
    for (int i = 1; i <= ntpguest; ++i)
      sum_za = sum_za + gstmolfract[i] * std::sqrt(ag[ig] * ag[i]) * (1 - kfug[ig][i]);
    const float sq2 = std::sqrt(2.0f);
    const double phi =
        std::exp(bg[ig] / bs * (z1 - 1) - std::log(z1 - B) -
                 as / (double(2.0f * sq2) * bs * R * temp) * (2 * sum_za / as - bg[ig] / bs) *
                     std::log((z1 + double(1.0f + sq2) * B) / (z1 + double(1.0f - sq2) * B)));
    gstfuga[ig] = phi * gstmolfract[ig] * gstpress[ig];
  }
}

// move-frequency normalisation (gcmc.f:341-386), REAL*4 arithmetic.
void Sim::normalise_moves() {
  for (int i = 1; i <= ntpguest; ++i) {
    mcmvnorm[i] = mcinsf[i] + mcdelf[i] + mcdisf[i] + mcjmpf[i] + mcswpf[i] +
                  mctraf[i] + mcrotf[i] + mcswif[i];
    if (mcmvnorm[i] == 0.0f) {
      mcmvnorm[i] = 1.0f;
      mcinsf[i] = (float)(1.0 / 3.0);
      mcdelf[i] = (float)(1.0 / 3.0);
      mcdisf[i] = (float)(1.0 / 3.0);
      mcjmpf[i] = mcswpf[i] = mctraf[i] = mcrotf[i] = mcswif[i] = 0.0f;
    }
    float nrm = mcmvnorm[i];
    mcinsf[i] = mcinsf[i] / nrm;
    mcdelf[i] = mcinsf[i] + (mcdelf[i] / nrm);
    mcdisf[i] = mcdelf[i] + (mcdisf[i] / nrm);
    mcjmpf[i] = mcdisf[i] + (mcjmpf[i] / nrm);
    mcswpf[i] = mcjmpf[i] + (mcswpf[i] / nrm);
    mctraf[i] = mcswpf[i] + (mctraf[i] / nrm);
    mcrotf[i] = mctraf[i] + (mcrotf[i] / nrm);
    mcswif[i] = mcrotf[i] + (mcswif[i] / nrm);
  }
}

// condense (utility_pack.f:3951-4050): guests first, then frameworks.
void Sim::condense() {
  size_t n = (size_t)totatm + 1;
  xxx.assign(n, 0.0);
  yyy.assign(n, 0.0);
  zzz.assign(n, 0.0);
  atmcharge.assign(n, 0.0);
  atmweight.assign(n, 0.0);
  ltype.assign(n, 0);
  moltype.assign(n, 0);
  lfreezesite.assign(n, 0);
  int jj = 0;
  auto put = [&](int mt) {
    MolType &m = mol[mt];
    int ii = 0;
    for (int im = 1; im <= m.nummols; ++im)
      for (int s = 1; s <= m.natoms; ++s) {
        ++ii;
        ++jj;
        xxx[jj] = m.mx[ii];
        yyy[jj] = m.my[ii];
        zzz[jj] = m.mz[ii];
        atmcharge[jj] = m.chg[s];
        lfreezesite[jj] = m.frz[s];
        atmweight[jj] = m.wght[s];
        ltype[jj] = m.ltp[s];
        moltype[jj] = mt;
      }
  };
  for (int g = 1; g <= ntpguest; ++g) put(locguest[g]);
  for (int fr = 1; fr <= ntpfram; ++fr) put(locfram[fr]);
  if (jj != totatm) fail("oracle: condense atom count mismatch");
}

// erfcgen (ewald.f:1-30): Abramowitz-Stegun 7.1.26 erfc(alpha r)/r table.
void Sim::erfcgen() {
  const double a1 = 0.254829592, a2 = -0.284496736, a3 = 1.421413741;
  const double a4 = -1.453152027, a5 = 1.061405429, pp = 0.3275911;
  erc.assign(mxegrd + 3, 0.0);
  fer.assign(mxegrd + 3, 0.0);
  if (keyfce / 2 == 1 || keyfce / 2 == 6) {
    drewd = rcut / double(mxegrd - 4);
    for (int i = 1; i <= mxegrd; ++i) {
      double rrr = double(i) * drewd;
      double rrrsq = rrr * rrr;
      double tt = 1.0 / (1.0 + pp * alpha * rrr);
      double ar = alpha * rrr;
      double exp1 = std::exp(-(ar * ar));
      erc[i] = tt * (a1 + tt * (a2 + tt * (a3 + tt * (a4 + tt * a5)))) * exp1 / rrr;
      fer[i] = erc[i] / rrrsq + 2.0 * (alpha / SQRPI) * exp1 / rrrsq;
    }
  }
}

// lrcorrect (vdw_terms.f:468-684; lj and 12-6 tails)
void Sim::lrcorrect() {
  int nmc = mxcmls();
  std::vector<double> elrc_mol0(nmc + 1, 0.0);
  double twopi = 2.0 * PI;
  elrc_mol.assign(nmc + 1, 0.0);
  numtyp.assign(mxatyp + 1, 0);
  numfrz.assign(mxatyp + 1, 0);
  numtyp_mol.assign(maxmls + 2, std::vector<int>(mxatyp + 1, 0));
  numfrz_mol.assign(maxmls + 2, std::vector<int>(mxatyp + 1, 0));
  numtyp_gstmol.assign(ntpguest + 1, std::vector<int>(mxatyp + 1, 0));
  numfrz_gstmol.assign(ntpguest + 1, std::vector<int>(mxatyp + 1, 0));
  for (int i = 1; i <= ntpguest; ++i) {
    int m = locguest[i];
    for (int j = 1; j <= mol[m].natoms; ++j) {
      int ka = mol[m].ltp[j];
      numtyp_gstmol[i][ka]++;
      if (mol[m].frz[j] != 0) numfrz_gstmol[i][ka]++;
    }
  }
  for (int i = 1; i <= totatm; ++i) {
    int ka = ltype[i];
    numtyp[ka]++;
    numtyp_mol[moltype[i]][ka]++;
    if (lfreezesite[i] != 0) {
      numfrz[ka]++;
      numfrz_mol[moltype[i]][ka]++;
    }
  }
  elrc = 0.0;
  steadd.assign(maxvdw + 2, 0.0);
  if (imcon != 0 && imcon != 6 && maxvdw > 0 && keyfce % 2 == 0) {
    int ivdw = 0;
    for (int i = 1; i <= ntpatm; ++i) {
      for (int j = 1; j <= i; ++j) {
        double eadd = 0.0;
        ++ivdw;
        int k = lstvdw[ivdw];
        if (ltpvdw[k] == 1) {
          double aaa = prmvdw[k][1], bbb = prmvdw[k][2];
          eadd = aaa / (9.0 * std::pow(rcut, 9)) - bbb / (3.0 * std::pow(rcut, 3));
        } else if (ltpvdw[k] == 2) {
          double e = prmvdw[k][1], s = prmvdw[k][2];
          eadd = 4.0 * e *
                 (std::pow(s, 12) / (9.0 * std::pow(rcut, 9)) -
                  std::pow(s, 6) / (3.0 * std::pow(rcut, 3)));
        }
        if (i != j) eadd *= 2.0;
        steadd[ivdw] = eadd;
        double denprd = twopi *
                        (double(numtyp[i]) * double(numtyp[j]) -
                         double(numfrz[i]) * double(numfrz[j])) /
                        (volm * volm);
        elrc = elrc + volm * denprd * eadd;
        std::fill(elrc_mol0.begin(), elrc_mol0.end(), 0.0);
        for (int it = 1; it <= maxmls; ++it)
          for (int jt = 1; jt <= maxmls; ++jt) {
            int kt = loc2(it, jt);
            double na = numtyp_mol[it][i], nb = numtyp_mol[jt][j];
            double fa = numfrz_mol[it][i], fb = numfrz_mol[jt][j];
            elrc_mol0[kt] += twopi * (na * nb - fa * fb) / (volm * volm);
          }
        for (int q = 1; q <= nmc; ++q) elrc_mol[q] += volm * eadd * elrc_mol0[q];
      }
    }
  }
}

// gstlrcorrect (vdw_terms.f:686-776)
void Sim::gstlrcorrect(int iguest, double &delrc, bool lexisting) {
  double twopi = 2.0 * PI;
  delrc = 0.0;
  int m = locguest[iguest];
  int nmc = mxcmls();
  if (imcon != 0 && imcon != 6 && maxvdw > 0 && keyfce % 2 == 0) {
    int ivdw = 0;
    for (int i = 1; i <= ntpatm; ++i) {
      for (int j = 1; j <= i; ++j) {
        ++ivdw;
        double eadd = steadd[ivdw];
        double na = numtyp_gstmol[iguest][i], nb = numtyp_gstmol[iguest][j];
        double fa = numfrz_gstmol[iguest][i], fb = numfrz_gstmol[iguest][j];
        double denprd = na * double(numtyp[j]) + nb * double(numtyp[i]) -
                        fa * double(numfrz[j]) - fb * double(numfrz[i]);
        if (lexisting) denprd = -1.0 * denprd;
        denprd = denprd + (na * nb - fa * fb);
        delrc = delrc + volm * twopi * denprd / (volm * volm) * eadd;
        std::fill(delrc_mol0.begin(), delrc_mol0.end(), 0.0);
        for (int jt = 1; jt <= maxmls; ++jt) {
          int kt = loc2(m, jt);
          double nc = numtyp_mol[jt][j], nd = numtyp_mol[jt][i];
          double fc = numfrz_mol[jt][j], fd = numfrz_mol[jt][i];
          double sic = na * nc + nb * nd - fa * fc - fb * fd;
          double self = 0.0;
          if (jt == m) {
            self = na * nb - fa * fb;
            if (lexisting) sic = -1.0 * sic;
          }
          delrc_mol0[kt] += twopi * (sic + self) / (volm * volm);
        }
        for (int q = 1; q <= nmc; ++q) delrc_mol[q] += volm * eadd * delrc_mol0[q];
      }
    }
  }
}

// ewald1 (ewald.f:354-661): full reciprocal sum, defines S(k) and newld.
void Sim::ewald1(double &engcpe, double &engsicold) {
  double twopi = 2.0 * PI;
  bool lconsw = true;
  engcpe = 0.0;
  int jj = 0;
  double rvolm = twopi / volm;
  double ralph = -0.25 / (alpha * alpha);
  if (imcon == 4 || imcon == 5 || imcon == 7) {
    rvolm = 0.5 * rvolm;
    lconsw = false;
  }
  double det, buffer[10];
  invert(cell, rcell, det);
  dcell(rcell, buffer);
  double rcpcut = std::fmin(double(kmax1) * buffer[6],
                            std::fmin(double(kmax2) * buffer[7],
                                      double(kmax3) * buffer[8]));
  rcpcut = rcpcut * 1.05 * twopi;
  double rcpct2 = rcpcut * rcpcut;
  int mxatm = totatm;
  engsicold = 0.0;
  for (int n = 1; n <= mxatm; ++n) {
    int m = moltype[n];
    double tchge = atmcharge[n] * atmcharge[n];
    int ik = loc2(m, m);
    engsicold += tchge;
    engsic[ik] += tchge;
    chgsum_mol[m] += atmcharge[n];
  }
  engsicold = -R4PIE0 / epsq * alpha * engsicold / SQRPI;
  // exponential factors (ewald.f:421-462)
  int limit = mxatm;
  int K2 = kmax2, K3 = kmax3;
  std::vector<double> elc0(limit + 1), els0(limit + 1), elc1(limit + 1),
      els1(limit + 1);
  std::vector<double> emc((size_t)(limit + 1) * (K2 + 1)),
      ems((size_t)(limit + 1) * (K2 + 1));
  std::vector<double> enc((size_t)(limit + 1) * (K3 + 1)),
      ens((size_t)(limit + 1) * (K3 + 1));
  auto EM = [&](std::vector<double> &v, int i, int l) -> double & {
    return v[(size_t)l * (limit + 1) + i];
  };
  for (int i = 1; i <= limit; ++i) {
    elc0[i] = 1.0;
    els0[i] = 0.0;
    EM(emc, i, 0) = 1.0;
    EM(ems, i, 0) = 0.0;
    EM(enc, i, 0) = 1.0;
    EM(ens, i, 0) = 0.0;
    double ssx = rcell[0] * xxx[i] + rcell[3] * yyy[i] + rcell[6] * zzz[i];
    double ssy = rcell[1] * xxx[i] + rcell[4] * yyy[i] + rcell[7] * zzz[i];
    double ssz = rcell[2] * xxx[i] + rcell[5] * yyy[i] + rcell[8] * zzz[i];
    elc1[i] = std::cos(twopi * ssx);
    if (K2 >= 1) EM(emc, i, 1) = std::cos(twopi * ssy);
    if (K3 >= 1) EM(enc, i, 1) = std::cos(twopi * ssz);
    els1[i] = std::sin(twopi * ssx);
    if (K2 >= 1) EM(ems, i, 1) = std::sin(twopi * ssy);
    if (K3 >= 1) EM(ens, i, 1) = std::sin(twopi * ssz);
  }
  for (int l = 2; l <= K2; ++l)
    for (int i = 1; i <= limit; ++i) {
      EM(emc, i, l) = EM(emc, i, l - 1) * EM(emc, i, 1) - EM(ems, i, l - 1) * EM(ems, i, 1);
      EM(ems, i, l) = EM(ems, i, l - 1) * EM(emc, i, 1) + EM(emc, i, l - 1) * EM(ems, i, 1);
    }
  for (int l = 2; l <= K3; ++l)
    for (int i = 1; i <= limit; ++i) {
      EM(enc, i, l) = EM(enc, i, l - 1) * EM(enc, i, 1) - EM(ens, i, l - 1) * EM(ens, i, 1);
      EM(ens, i, l) = EM(ens, i, l - 1) * EM(enc, i, 1) + EM(enc, i, l - 1) * EM(ens, i, 1);
    }
  std::vector<double> clm(limit + 1), slm(limit + 1), ckcv(limit + 1),
      cksv(limit + 1);
  int kkk = 0, mmin = 0, nmin = 1;
  std::vector<double> &e1 = ewald1en;
  for (int ll = 0; ll <= kmax1; ++ll) {
    int l = ll;
    double tmp = twopi * double(ll);
    double rkx1 = tmp * rcell[0], rky1 = tmp * rcell[3], rkz1 = tmp * rcell[6];
    if (l == 1) {
      for (int i = 1; i <= limit; ++i) {
        elc0[i] = elc1[i];
        els0[i] = els1[i];
      }
    } else if (l > 1) {
      for (int i = 1; i <= limit; ++i) {
        double cs = elc0[i];
        elc0[i] = cs * elc1[i] - els0[i] * els1[i];
        els0[i] = els0[i] * elc1[i] + cs * els1[i];
      }
    }
    for (int mm = mmin; mm <= kmax2; ++mm) {
      int m = std::abs(mm);
      double t2 = twopi * double(mm);
      double rkx2 = rkx1 + t2 * rcell[1], rky2 = rky1 + t2 * rcell[4],
             rkz2 = rkz1 + t2 * rcell[7];
      if (mm >= 0) {
        for (int i = 1; i <= limit; ++i) {
          clm[i] = elc0[i] * EM(emc, i, m) - els0[i] * EM(ems, i, m);
          slm[i] = els0[i] * EM(emc, i, m) + EM(ems, i, m) * elc0[i];
        }
      } else {
        for (int i = 1; i <= limit; ++i) {
          clm[i] = elc0[i] * EM(emc, i, m) + els0[i] * EM(ems, i, m);
          slm[i] = els0[i] * EM(emc, i, m) - EM(ems, i, m) * elc0[i];
        }
      }
      for (int nn = nmin; nn <= kmax3; ++nn) {
        int n = std::abs(nn);
        double t3 = twopi * double(nn);
        double rkx3 = rkx2 + t3 * rcell[2], rky3 = rky2 + t3 * rcell[5],
               rkz3 = rkz2 + t3 * rcell[8];
        double rksq = rkx3 * rkx3 + rky3 * rky3 + rkz3 * rkz3;
        if (rksq <= rcpct2) {
          for (int i = 1; i <= limit; ++i) {
            double tchge = atmcharge[i], tclm = clm[i], tenc = EM(enc, i, n),
                   tslm = slm[i], tens = EM(ens, i, n);
            if (nn >= 0) {
              ckcv[i] = tchge * (tclm * tenc - tslm * tens);
              cksv[i] = tchge * (tslm * tenc + tclm * tens);
            } else {
              ckcv[i] = tchge * (tclm * tenc + tslm * tens);
              cksv[i] = tchge * (tslm * tenc - tclm * tens);
            }
          }
          double ckcs = 0.0, ckss = 0.0;
          ++jj;
          ++kkk;
          if (kkk > mxebuf) fail("oracle: k-vector buffer overflow");
          for (int i = 1; i <= limit; ++i) {
            ckcs += ckcv[i];
            ckss += cksv[i];
            int mt = moltype[i];
            ckc(ckcsum, mt, kkk) += ckcv[i];
            ckc(ckssum, mt, kkk) += cksv[i];
            ckc(ckcsum, maxmls + 1, kkk) += ckcv[i];
            ckc(ckssum, maxmls + 1, kkk) += cksv[i];
          }
          double rrksq = 1.0 / rksq;
          double akk = lconsw ? std::exp(ralph * rksq) * rrksq
                              : 4.0 * std::exp(ralph * rksq) * rrksq;
          engcpe = engcpe + akk * (ckcs * ckcs + ckss * ckss);
          int kmol = 0;
          for (int i = 1; i <= maxmls; ++i) {
            double fkk = 2.0 * akk;
            for (int j = 1; j <= i; ++j) {
              ++kmol;
              if (i == j) fkk = akk;
              e1[kmol] += fkk * (ckc(ckcsum, i, kkk) * ckc(ckcsum, j, kkk) +
                                 ckc(ckssum, i, kkk) * ckc(ckssum, j, kkk));
            }
          }
        }
      }
      nmin = -kmax3;
    }
    mmin = -kmax2;
  }
  newld = jj;
  double qfix = -(0.5 * PI * R4PIE0 / epsq) * ((sumchg / alpha) * (sumchg / alpha) / volm);
  double rv = lconsw ? 2.0 * rvolm : rvolm;
  engcpe = rv * R4PIE0 * engcpe / epsq + engsicold + qfix;
  for (int i = 1; i <= maxmls; ++i) {
    double fkk = 1.0;
    for (int j = 1; j <= i; ++j) {
      if (i == j) fkk = 0.5;
      int ik = loc2(i, j);
      double sic = -R4PIE0 / epsq * alpha * engsic[ik] / SQRPI;
      sic = sic - ((fkk * PI * R4PIE0 / epsq) * chgsum_mol[i] * chgsum_mol[j] /
                   (alpha * alpha * volm));
      e1[ik] = rv * R4PIE0 * e1[ik] / epsq + sic;
    }
  }
}

// ewald1_guest (ewald.f:32-352): reciprocal energy of one guest.
void Sim::ewald1_guest(double &engcpe, int natms, int iguest, double &chgtmp,
                       double &engsictmp, bool lexisting) {
  double twopi = 2.0 * PI;
  bool lconsw = true;
  engcpe = 0.0;
  int m0 = locguest[iguest];
  for (int ik = 1; ik <= newld; ++ik) {
    ckc(ckcsnew, m0, ik) = 0.0;
    ckc(ckssnew, m0, ik) = 0.0;
    ckc(ckcsnew, maxmls + 1, ik) = 0.0;
    ckc(ckssnew, maxmls + 1, ik) = 0.0;
  }
  double rvolm = twopi / volm;
  double ralph = -0.25 / (alpha * alpha);
  if (imcon == 4 || imcon == 5 || imcon == 7) {
    rvolm = 0.5 * rvolm;
    lconsw = false;
  }
  double det, buffer[10];
  invert(cell, rcell, det);
  dcell(rcell, buffer);
  double rcpcut = std::fmin(double(kmax1) * buffer[6],
                            std::fmin(double(kmax2) * buffer[7],
                                      double(kmax3) * buffer[8]));
  rcpcut = rcpcut * 1.05 * twopi;
  double rcpct2 = rcpcut * rcpcut;
  chgtmp = 0.0;
  engsictmp = 0.0;
  for (int n = 1; n <= natms; ++n) {
    double chge = mol[m0].chg[n];
    chgtmp += chge;
    engsictmp += chge * chge;
  }
  engsictmp = -R4PIE0 / epsq * alpha * engsictmp / SQRPI;
  int limit = natms;
  int K2 = kmax2, K3 = kmax3;
  std::vector<double> elc0(limit + 1), els0(limit + 1), elc1(limit + 1),
      els1(limit + 1), emc((limit + 1) * (K2 + 1)), ems((limit + 1) * (K2 + 1)),
      enc((limit + 1) * (K3 + 1)), ens((limit + 1) * (K3 + 1));
  auto EM = [&](std::vector<double> &v, int i, int l) -> double & {
    return v[(size_t)l * (limit + 1) + i];
  };
  for (int i = 1; i <= limit; ++i) {
    elc0[i] = 1.0;
    els0[i] = 0.0;
    EM(emc, i, 0) = 1.0;
    EM(ems, i, 0) = 0.0;
    EM(enc, i, 0) = 1.0;
    EM(ens, i, 0) = 0.0;
    double ssx = rcell[0] * newx[i] + rcell[3] * newy[i] + rcell[6] * newz[i];
    double ssy = rcell[1] * newx[i] + rcell[4] * newy[i] + rcell[7] * newz[i];
    double ssz = rcell[2] * newx[i] + rcell[5] * newy[i] + rcell[8] * newz[i];
    elc1[i] = std::cos(twopi * ssx);
    if (K2 >= 1) EM(emc, i, 1) = std::cos(twopi * ssy);
    if (K3 >= 1) EM(enc, i, 1) = std::cos(twopi * ssz);
    els1[i] = std::sin(twopi * ssx);
    if (K2 >= 1) EM(ems, i, 1) = std::sin(twopi * ssy);
    if (K3 >= 1) EM(ens, i, 1) = std::sin(twopi * ssz);
  }
  for (int l = 2; l <= K2; ++l)
    for (int i = 1; i <= limit; ++i) {
      EM(emc, i, l) = EM(emc, i, l - 1) * EM(emc, i, 1) - EM(ems, i, l - 1) * EM(ems, i, 1);
      EM(ems, i, l) = EM(ems, i, l - 1) * EM(emc, i, 1) + EM(emc, i, l - 1) * EM(ems, i, 1);
    }
  for (int l = 2; l <= K3; ++l)
    for (int i = 1; i <= limit; ++i) {
      EM(enc, i, l) = EM(enc, i, l - 1) * EM(enc, i, 1) - EM(ens, i, l - 1) * EM(ens, i, 1);
      EM(ens, i, l) = EM(ens, i, l - 1) * EM(enc, i, 1) + EM(enc, i, l - 1) * EM(ens, i, 1);
    }
  std::vector<double> clm(limit + 1), slm(limit + 1), ckcv(limit + 1),
      cksv(limit + 1);
  int kkk = 0, mmin = 0, nmin = 1;
  for (int ll = 0; ll <= kmax1; ++ll) {
    int l = ll;
    double tmp = twopi * double(ll);
    double rkx1 = tmp * rcell[0], rky1 = tmp * rcell[3], rkz1 = tmp * rcell[6];
    if (l == 1) {
      for (int i = 1; i <= limit; ++i) {
        elc0[i] = elc1[i];
        els0[i] = els1[i];
      }
    } else if (l > 1) {
      for (int i = 1; i <= limit; ++i) {
        double cs = elc0[i];
        elc0[i] = cs * elc1[i] - els0[i] * els1[i];
        els0[i] = els0[i] * elc1[i] + cs * els1[i];
      }
    }
    for (int mm = mmin; mm <= kmax2; ++mm) {
      int m = std::abs(mm);
      double t2 = twopi * double(mm);
      double rkx2 = rkx1 + t2 * rcell[1], rky2 = rky1 + t2 * rcell[4],
             rkz2 = rkz1 + t2 * rcell[7];
      if (mm >= 0) {
        for (int i = 1; i <= limit; ++i) {
          clm[i] = elc0[i] * EM(emc, i, m) - els0[i] * EM(ems, i, m);
          slm[i] = els0[i] * EM(emc, i, m) + EM(ems, i, m) * elc0[i];
        }
      } else {
        for (int i = 1; i <= limit; ++i) {
          clm[i] = elc0[i] * EM(emc, i, m) + els0[i] * EM(ems, i, m);
          slm[i] = els0[i] * EM(emc, i, m) - EM(ems, i, m) * elc0[i];
        }
      }
      for (int nn = nmin; nn <= kmax3; ++nn) {
        int n = std::abs(nn);
        double t3 = twopi * double(nn);
        double rkx3 = rkx2 + t3 * rcell[2], rky3 = rky2 + t3 * rcell[5],
               rkz3 = rkz2 + t3 * rcell[8];
        double rksq = rkx3 * rkx3 + rky3 * rky3 + rkz3 * rkz3;
        if (rksq <= rcpct2) {
          for (int i = 1; i <= limit; ++i) {
            double tchge = mol[m0].chg[i], tclm = clm[i], tenc = EM(enc, i, n),
                   tslm = slm[i], tens = EM(ens, i, n);
            if (nn >= 0) {
              ckcv[i] = tchge * (tclm * tenc - tslm * tens);
              cksv[i] = tchge * (tslm * tenc + tclm * tens);
            } else {
              ckcv[i] = tchge * (tclm * tenc + tslm * tens);
              cksv[i] = tchge * (tslm * tenc - tclm * tens);
            }
          }
          double ckcs = 0.0, ckss = 0.0;
          for (int i = 1; i <= limit; ++i) {
            ckcs += ckcv[i];
            ckss += cksv[i];
          }
          ++kkk;
          double ckcold = ckc(ckcsum, maxmls + 1, kkk);
          double cksold = ckc(ckssum, maxmls + 1, kkk);
          ckc(ckcsnew, m0, kkk) += ckcs;
          ckc(ckssnew, m0, kkk) += ckss;
          ckc(ckcsnew, maxmls + 1, kkk) += ckcs;
          ckc(ckssnew, maxmls + 1, kkk) += ckss;
          double rrksq = 1.0 / rksq;
          double akk = lconsw ? std::exp(ralph * rksq) * rrksq
                              : 4.0 * std::exp(ralph * rksq) * rrksq;
          double sumsqd = ckcs * ckcs + ckss * ckss;
          double mixterm = 2.0 * ckcs * ckcold + 2.0 * ckss * cksold;
          if (lexisting) mixterm = -1.0 * mixterm;
          engcpe = engcpe + akk * (mixterm + sumsqd);
          for (int i = 1; i <= maxmls; ++i) {
            double fkk = 2.0 * akk;
            if (i == m0) fkk = akk;
            int kmol = loc2(i, m0);
            ewald1en[kmol] += fkk * (ckc(ckcsnew, m0, kkk) * ckc(ckcsum, i, kkk) +
                                     ckc(ckssnew, m0, kkk) * ckc(ckssum, i, kkk));
          }
        }
      }
      nmin = -kmax3;
    }
    mmin = -kmax2;
  }
  double qfix = -(0.5 * PI * R4PIE0 / epsq) *
                ((chgtmp * sumchg) / alpha + (chgtmp / alpha) * (chgtmp / alpha)) / volm;
  if (lexisting) {
    engsictmp = -engsictmp;
    qfix = -qfix;
  }
  engcpe = 2.0 * rvolm * R4PIE0 * engcpe / epsq + engsictmp + qfix;
  for (int i = 1; i <= maxmls; ++i) {
    double fkk = 1.0, sic = 0.0;
    if (i == m0) {
      fkk = 0.5;
      sic = engsictmp;
    }
    double qfixmol = -(fkk * PI * R4PIE0 / epsq) * (chgsum_mol[i] * chgtmp) /
                     (alpha * alpha * volm);
    if (lexisting) {
      sic = -sic;
      qfixmol = -qfixmol;
    }
    int kmol = loc2(i, m0);
    ewald1en[kmol] = 2.0 * rvolm * R4PIE0 * ewald1en[kmol] / epsq + sic + qfixmol;
  }
}

// ewald2 (ewald.f:663-733): real-space erfc term, 3-point interpolation.
void Sim::ewald2(double chg, int natm, double &engcpe, int molt) {
  double rcsq = rcut * rcut;
  double rdrewd = 1.0 / drewd;
  engcpe = 0.0;
  double chgea = chg / epsq * R4PIE0;
  for (int i = 1; i <= natm; ++i) {
    int jatm = ilist[i];
    int jmol = moldf[i];
    double chgprd = chgea * atmcharge[jatm];
    if (std::fabs(chgprd) > 1.0e-10) {
      double rsq = rsqdf[i];
      if (rcsq > rsq) {
        double rrr = std::sqrt(rsq);
        int ll = int(rrr * rdrewd);
        if (ll < 1) fail("oracle: erfc table index below 1 (pair closer than the grid step)");
        int l1 = ll + 1, l2 = ll + 2;
        double ppp = rrr * rdrewd - double(ll);
        double vk0 = erc[ll], vk1 = erc[l1], vk2 = erc[l2];
        double t1 = vk0 + (vk1 - vk0) * ppp;
        double t2 = vk1 + (vk2 - vk1) * (ppp - 1.0);
        double erfcr = (t1 + (t2 - t1) * ppp * 0.5) * chgprd;
        engcpe = engcpe + erfcr;
        ewald2en[loc2(molt, jmol)] += erfcr;
      }
    }
  }
}

// ewald3 (ewald.f:735-790): erfc-complement correction of excluded pairs.
void Sim::ewald3(double chg, int molt, int natms, const std::vector<int> &jlist,
                 double &engcpe) {
  const double a1 = 0.254829592, a2 = -0.284496736, a3 = 1.421413741;
  const double a4 = -1.453152027, a5 = 1.061405429, pp = 0.3275911;
  const double rr3 = 0.333333333333, r10 = 0.1, r42 = 0.02380952381,
               r216 = 4.62962962963e-3;
  engcpe = 0.0;
  double chgea = chg / epsq * R4PIE0;
  for (int m = 1; m <= natms; ++m) {
    int jatm = jlist[m];
    double chgprd = chgea * mol[molt].chg[jatm];
    double rsq = xdf[m] * xdf[m] + ydf[m] * ydf[m] + zdf[m] * zdf[m];
    double rrr = std::sqrt(rsq);
    double alpr = rrr * alpha;
    double alpr2 = alpr * alpr;
    double erfr;
    if (alpr < 1.0e-2) {
      erfr = 2.0 * chgprd * (alpha / SQRPI) *
             (1.0 + alpr2 * (-rr3 + alpr2 * (r10 + alpr2 * (-r42 + alpr2 * r216))));
    } else {
      double tt = 1.0 / (1.0 + pp * alpha * rrr);
      double ar = alpha * rrr;
      double exp1 = std::exp(-(ar * ar));
      erfr = (1.0 - tt * (a1 + tt * (a2 + tt * (a3 + tt * (a4 + tt * a5)))) * exp1) *
             chgprd / rrr;
    }
    engcpe = engcpe + erfr;
  }
}

// srfrce (vdw_terms.f:382-466): tabulated van der Waals, 3-point interpolation.
void Sim::srfrce(int sittyp, int ik, int molt, double &engsrp) {
  double rcsq = rcut * rcut;
  double rdr = 1.0 / dlrpot;
  engsrp = 0.0;
  double ai = double(sittyp);
  for (int m = 1; m <= ik; ++m) {
    int jatm = ilist[m];
    int jmol = moldf[m];
    double aj = double(ltype[jatm]);
    double ab;
    if (ai > aj)
      ab = ai * (ai - 1.0) * 0.5 + aj + 0.5;
    else
      ab = aj * (aj - 1.0) * 0.5 + ai + 0.5;
    int k = lstvdw[int(ab)];
    if (ltpvdw[k] < 100 && std::fabs(vvv[k][1]) > 1.0e-10) {
      double rsq = rsqdf[m];
      if (rcsq > rsq) {
        double rrr = std::sqrt(rsq);
        int l = int(rrr * rdr);
        if (l < 1) fail("oracle: vdw table index below 1 (pair closer than the grid step)");
        double ppp = rrr * rdr - double(l);
        double vk0 = vvv[k][l], vk1 = vvv[k][l + 1], vk2 = vvv[k][l + 2];
        double t1 = vk0 + (vk1 - vk0) * ppp;
        double t2 = vk1 + (vk2 - vk1) * (ppp - 1.0);
        double omega = t1 + (t2 - t1) * ppp * 0.5;
        engsrp = omega + engsrp;
        vdwen[loc2(jmol, molt)] += omega;
      }
    }
  }
}

// excluding_ewald_charges (gcmc.f:2662-2761), guest molecules.  The
// framework branch of the reference adds nothing to the totals it returns.
void Sim::excluding_ewald_charges(double &ewald3sum) {
  ewald3sum = 0.0;
  std::fill(ewald3en.begin(), ewald3en.end(), 0.0);
  for (int m = 1; m <= ntpmls; ++m) {
    double ewald3mol = 0.0;
    for (int ig = 1; ig <= ntpguest; ++ig) {
      if (locguest[ig] != m) continue;
      int natms = mol[m].natoms;
      for (int iatm = 1; iatm <= natms - 1; ++iatm) {
        int ik = 0;
        std::vector<int> jlist(natms + 1, 0);
        xdf.assign(natms + 1, 0.0);
        ydf.assign(natms + 1, 0.0);
        zdf.assign(natms + 1, 0.0);
        for (int jatm = iatm + 1; jatm <= natms; ++jatm) {
          ++ik;
          jlist[ik] = jatm;
          xdf[ik] = guestx[ig][iatm] - guestx[ig][jatm];
          ydf[ik] = guesty[ig][iatm] - guesty[ig][jatm];
          zdf[ik] = guestz[ig][iatm] - guestz[ig][jatm];
        }
        images(imcon, ik, cell, &xdf[1], &ydf[1], &zdf[1]);
        double e;
        ewald3(mol[m].chg[iatm], m, ik, jlist, e);
        ewald3mol += e;
        ewald3en[m] += e;
      }
      ewald3sum += mol[m].nummols * ewald3mol;
    }
  }
}

// single_point (gcmc.f:2549-2660) for a frozen framework without guests:
// every framework pair is excluded by parlst (nlist_builders.f:120), so the
// real-space and van der Waals sums vanish.
void Sim::single_point() {
  int nmc = mxcmls();
  vdwen.assign(nmc + 2, 0.0);
  ewald2en.assign(nmc + 2, 0.0);
  ewald1en.assign(nmc + 2, 0.0);
  ewald3en.assign(maxmls + 2, 0.0);
  delrc_mol.assign(nmc + 2, 0.0);
  delrc_mol0.assign(nmc + 2, 0.0);
  for (int m = 1; m <= maxmls; ++m) {
    if (!mol[m].guest) {
      for (int s = 1; s <= mol[m].natoms; ++s)
        if (mol[m].frz[s] == 0)
          fail("oracle: non-frozen framework atoms are not restated");
    } else if (mol[m].nummols > 0) {
      fail("oracle: guests present in CONFIG are not restated (use create molecules)");
    }
  }
  lrcorrect();
  condense();
  double engsicold;
  ewald1(ewald1sum, engsicold);
  double ewald3eng;
  excluding_ewald_charges(ewald3eng);
  double ewald2sum = 0.0, vdwsum = 0.0;
  spe_dlpeng = ewald1sum + ewald2sum + vdwsum - ewald3eng + elrc;
  spe_ecoul = ewald2sum + ewald1sum - ewald3eng;
  spe_vdw = (vdwsum + elrc) / engunit;
  // initial guest energies (gcmc.f:549-583)
  for (int ig = 1; ig <= ntpguest; ++ig) {
    int m = locguest[ig];
    double spenergy = 0.0;
    for (int jm = 1; jm <= ntpmls; ++jm) {
      int ik = loc2(m, jm);
      spenergy += (ewald1en[ik] + ewald2en[ik] + elrc_mol[ik] + vdwen[ik]) / engunit;
    }
    if (mol[m].nummols > 0) spenergy -= mol[m].nummols * ewald3en[m] / engunit;
    energy[m] = spenergy;
  }
}

void Sim::read_all(const std::string &dir) {
  initscan(dir);
  // alloc_config_arrays defaults (utility_pack.f:1139-1200)
  mcinsf.assign(maxmls + 1, -1.0f);
  mcdelf = mcdisf = mcjmpf = mcswpf = mctraf = mcrotf = mcswif = mcinsf;
  mcmvnorm.assign(maxmls + 1, 0.0f);
  guest_insert.assign(maxmls + 1, 0);
  readfield(dir);
  readconfig(dir);
  int nmc = mxcmls();
  mxebuf = (2 * kmax1 + 1) * (2 * kmax2 + 1) * (2 * kmax3 + 1) - 1;
  size_t nsk = (size_t)(maxmls + 1) * mxebuf;
  ckcsum.assign(nsk, 0.0);
  ckssum.assign(nsk, 0.0);
  ckcsnew.assign(nsk, 0.0);
  ckssnew.assign(nsk, 0.0);
  ckcsorig.assign(nsk, 0.0);
  ckssorig.assign(nsk, 0.0);
  ewald1en.assign(nmc + 2, 0.0);
  ewald1entmp.assign(nmc + 2, 0.0);
  ewald2en.assign(nmc + 2, 0.0);
  ewald2entmp.assign(nmc + 2, 0.0);
  ewald3en.assign(maxmls + 2, 0.0);
  engsic.assign(nmc + 2, 0.0);
  engsicorig.assign(nmc + 2, 0.0);
  chgsum_mol.assign(maxmls + 2, 0.0);
  vdwentmp.assign(nmc + 2, 0.0);
  statvolm = volm * 1e-30;
  double det;
  invert(cell, rcell, det);
  setup_grid();
  delr.assign(ntpguest + 1, initdelr);
  disp_ratio.assign(ntpguest + 1, 0.5);
  tran_ratio.assign(ntpguest + 1, 0.5);
  rota_ratio.assign(ntpguest + 1, 0.5);
  readcontrol(dir);
  overlap = overlap * overlap;
  fugacity();
  normalise_moves();
  delE.assign(nmc + 2, 0.0);
  energy.assign(maxmls + 2, 0.0);
  surfacemols.assign(maxmls + 2, 0.0);
  int ng = ntpguest + 1;
  ins_count.assign(ng, 0);
  accept_ins = del_count = accept_del = disp_count = accept_disp = tran_count =
      accept_tran = rota_count = accept_rota = jump_count = accept_jump = swap_count =
          accept_swap = switch_count = accept_switch = ins_count;
  condense();  // gcmc.f:515-516
  beta = 1.0 / (KBOLTZ * temp);
  epsq = 1.0;
  erfcgen();
  single_point();
  chainstats.assign(1 + 16 * ntpguest + 1, 0.0);
  delrdisp = delr;
  tran_delr = delr;
  rotangle = PI / 3.0;
  rota_rotangle = rotangle;
  minchk = std::min(400, nnumg);
  if (minchk < 1) minchk = 1;
  production = (eqsteps == 0);
  int mxg = 50;
  newx.assign(mxg + 1, 0.0);
  newy.assign(mxg + 1, 0.0);
  newz.assign(mxg + 1, 0.0);
  ind.assign(mxg + 1, 0);
}

}  // namespace

namespace {
// guestlistgen (utility_pack.f:3711-3774): brute-force per-site list of
// all atoms except the guest's own (ind), radius rcut+ddelr.
void guestlistgen_r(Sim &S, int natms, double ddelr) {
  double rclim = (S.rcut + ddelr) * (S.rcut + ddelr);
  int tot = S.totatm;
  if ((int)S.xdf.size() < tot + 1) {
    S.xdf.assign(tot + 1, 0.0);
    S.ydf.assign(tot + 1, 0.0);
    S.zdf.assign(tot + 1, 0.0);
  }
  S.gstlentry.assign(natms + 1, 0);
  S.gstlist.assign(natms + 1, std::vector<int>());
  for (int i = 1; i <= natms; ++i) {
    int ii = 0;
    for (int j = 1; j <= tot; ++j) {
      bool chk = true;
      for (int it = 1; it <= natms; ++it)
        if (j == S.ind[it]) chk = false;
      if (chk) {
        ++ii;
        S.xdf[ii] = S.newx[i] - S.xxx[j];
        S.ydf[ii] = S.newy[i] - S.yyy[j];
        S.zdf[ii] = S.newz[i] - S.zzz[j];
      }
    }
    images(S.imcon, ii, S.cell, &S.xdf[1], &S.ydf[1], &S.zdf[1]);
    ii = 0;
    for (int j = 1; j <= tot; ++j) {
      bool chk = true;
      for (int it = 1; it <= natms; ++it)
        if (j == S.ind[it]) chk = false;
      if (chk) {
        ++ii;
        double rsq = S.xdf[ii] * S.xdf[ii] + S.ydf[ii] * S.ydf[ii] +
                     (S.imcon == 6 ? 0.0 : S.zdf[ii] * S.zdf[ii]);
        if (rsq <= rclim) {
          S.gstlentry[i]++;
          S.gstlist[i].push_back(j);
        }
      }
    }
  }
}
}  // namespace

namespace {

// surface_check (mc_moves.f:10-44)
void Sim::surface_check(int iatm, int j, int molt, bool &loverlap,
                        bool &latmsurf) {
  latmsurf = false;
  int jatm = ilist[j];
  int aa = mol[molt].ltp[iatm];
  int ab = ltype[jatm];
  double ak;
  if (aa > ab)
    ak = aa * (aa - 1.0) * 0.5 + ab + 0.5;
  else
    ak = ab * (ab - 1.0) * 0.5 + aa + 0.5;
  int ivdw = lstvdw[int(ak)];
  double sig = prmvdw[ivdw][2];
  double req = sig;
  double st = surftol + req;
  double surftolsq = st * st;
  if (rsqdf[j] < surftolsq && lfreezesite[jatm] == 1) latmsurf = true;
  if (rsqdf[j] < overlap) loverlap = true;
}

// Fill the per-site pair arrays for guest site i (mc_moves.f:202-216).
void fill_site(Sim &S, int i) {
  int n = S.gstlentry[i];
  if ((int)S.ilist.size() < n + 1) {
    S.ilist.assign(n + 1, 0);
    S.moldf.assign(n + 1, 0);
  }
  if ((int)S.rsqdf.size() < n + 1) S.rsqdf.assign(n + 1, 0.0);
  if ((int)S.xdf.size() < n + 1) {
    S.xdf.assign(n + 1, 0.0);
    S.ydf.assign(n + 1, 0.0);
    S.zdf.assign(n + 1, 0.0);
  }
  for (int j = 1; j <= n; ++j) {
    int jatm = S.gstlist[i][j - 1];
    S.ilist[j] = jatm;
    S.moldf[j] = S.moltype[jatm];
    S.xdf[j] = S.newx[i] - S.xxx[jatm];
    S.ydf[j] = S.newy[i] - S.yyy[jatm];
    S.zdf[j] = S.newz[i] - S.zzz[jatm];
  }
  images(S.imcon, n, S.cell, &S.xdf[1], &S.ydf[1], &S.zdf[1]);
}

// insertion (mc_moves.f:150-276)
void Sim::insertion(int iguest, double &delrc, double &estep, double &chgtmp,
                    double &engsictmp, bool &loverlap, bool &lnewsurf,
                    double *parts) {
  int m0 = locguest[iguest];
  int nmc = mxcmls();
  lnewsurf = false;
  bool latmsurf = false;
  loverlap = false;
  int natms = mol[m0].natoms;
  double ewld2sum = 0.0, vdwsum = 0.0;
  std::fill(ind.begin(), ind.end(), 0);
  for (int ik = 1; ik <= nmc; ++ik) {
    delE[ik] = 0.0;
    ewald1en[ik] = 0.0;
    ewald2en[ik] = 0.0;
    vdwen[ik] = 0.0;
    delrc_mol[ik] = 0.0;
  }
  guestlistgen_r(*this, natms, delr[iguest]);
  gstlrcorrect(iguest, delrc, false);
  for (int i = 1; i <= natms; ++i) {
    fill_site(*this, i);
    for (int l = 1; l <= gstlentry[i]; ++l) {
      rsqdf[l] = xdf[l] * xdf[l] + ydf[l] * ydf[l] + zdf[l] * zdf[l];
      surface_check(i, l, m0, loverlap, latmsurf);
      if (latmsurf) lnewsurf = true;
      if (loverlap) return;
    }
    double chg = mol[m0].chg[i];
    int sittyp = mol[m0].ltp[i];
    double e2, ev;
    ewald2(chg, gstlentry[i], e2, m0);
    ewld2sum += e2;
    srfrce(sittyp, gstlentry[i], m0, ev);
    vdwsum += ev;
  }
  engsictmp = 0.0;
  chgtmp = 0.0;
  double ewld1eng;
  ewald1_guest(ewld1eng, natms, iguest, chgtmp, engsictmp, false);
  double ewld3sum = ewald3en[m0];
  estep = estep + (ewld1eng + ewld2sum - ewld3sum + vdwsum + delrc) / engunit;
  for (int i = 1; i <= maxmls; ++i) {
    int ik = loc2(m0, i);
    double d = delrc_mol[ik];
    if (i != m0) delE[i] += (ewald1en[ik] + ewald2en[ik] + vdwen[ik] + d) / engunit;
  }
  delE[m0] += estep;
  if (parts) {
    parts[0] = ewld1eng;
    parts[1] = ewld2sum;
    parts[2] = vdwsum;
  }
}

// guest_energy (mc_moves.f:277-374)
void Sim::guest_energy(int iguest, double &vdwsum, double &ewld2sum,
                       double &ewld1eng, bool &lsurf, double &chgtmp,
                       double &engsictmp, bool &loverlap, double &estep,
                       bool lexisting) {
  int m0 = locguest[iguest];
  int natms = mol[m0].natoms;
  int nmc = mxcmls();
  ewld2sum = 0.0;
  vdwsum = 0.0;
  lsurf = false;
  loverlap = false;
  bool latmsurf = false;
  for (int ik = 1; ik <= nmc; ++ik) {
    delE[ik] = 0.0;
    ewald1en[ik] = 0.0;
    ewald2en[ik] = 0.0;
    vdwen[ik] = 0.0;
    delrc_mol[ik] = 0.0;
  }
  guestlistgen_r(*this, natms, delr[iguest]);
  estep = 0.0;
  chgtmp = 0.0;
  engsictmp = 0.0;
  ewald1_guest(ewld1eng, natms, iguest, chgtmp, engsictmp, lexisting);
  for (int i = 1; i <= natms; ++i) {
    int itatm = ind[i];
    fill_site(*this, i);
    for (int l = 1; l <= gstlentry[i]; ++l) {
      rsqdf[l] = xdf[l] * xdf[l] + ydf[l] * ydf[l] + zdf[l] * zdf[l];
      surface_check(i, l, m0, loverlap, latmsurf);
      if (latmsurf) lsurf = true;
      if (loverlap) return;
    }
    double chg = atmcharge[itatm];
    int sittyp = ltype[itatm];
    double e2, ev;
    ewald2(chg, gstlentry[i], e2, m0);
    ewld2sum += e2;
    srfrce(sittyp, gstlentry[i], m0, ev);
    vdwsum += ev;
  }
  double ewld3sum = ewald3en[m0];
  if (lexisting)
    estep = (-ewld1eng + ewld2sum + vdwsum - ewld3sum) / engunit;
  else
    estep = (ewld1eng + ewld2sum + vdwsum - ewld3sum) / engunit;
}

// get_guest (utility_pack.f:3776-3807)
void Sim::get_guest(int iguest, int choice, int &molt, int &natms, int &nmols) {
  molt = locguest[iguest];
  natms = mol[molt].natoms;
  nmols = mol[molt].nummols;
  int atmadd = 0;
  for (int i = 1; i <= iguest - 1; ++i) {
    int im = locguest[i];
    atmadd += mol[im].natoms * mol[im].nummols;
  }
  int at = (choice - 1) * natms + 1;
  int iatm = 0;
  for (int i = at; i <= at - 1 + natms; ++i) {
    ++iatm;
    ind[iatm] = atmadd + i;
    newx[iatm] = mol[molt].mx[i];
    newy[iatm] = mol[molt].my[i];
    newz[iatm] = mol[molt].mz[i];
  }
}

// deletion (mc_moves.f:375-484)
void Sim::deletion(int iguest, int choice, double &delrc, double &estep,
                   bool &linitsurf, double &engsictmp, double &chgtmp,
                   double *parts) {
  double ewld2sum = 0.0, vdwsum = 0.0;
  int m0, natms, nmols;
  get_guest(iguest, choice, m0, natms, nmols);
  linitsurf = false;
  bool loverlap = false, latmsurf = false;
  int nmc = mxcmls();
  for (int ik = 1; ik <= nmc; ++ik) {
    delE[ik] = 0.0;
    ewald1en[ik] = 0.0;
    ewald2en[ik] = 0.0;
    vdwen[ik] = 0.0;
    delrc_mol[ik] = 0.0;
  }
  gstlrcorrect(iguest, delrc, true);
  guestlistgen_r(*this, natms, delr[iguest]);
  estep = 0.0;
  chgtmp = 0.0;
  engsictmp = 0.0;
  double ewld1eng;
  ewald1_guest(ewld1eng, natms, iguest, chgtmp, engsictmp, true);
  for (int i = 1; i <= natms; ++i) {
    int itatm = ind[i];
    fill_site(*this, i);
    for (int l = 1; l <= gstlentry[i]; ++l) {
      rsqdf[l] = xdf[l] * xdf[l] + ydf[l] * ydf[l] + zdf[l] * zdf[l];
      surface_check(i, l, m0, loverlap, latmsurf);
      if (latmsurf) linitsurf = true;
    }
    double chg = atmcharge[itatm];
    int sittyp = ltype[itatm];
    double e2, ev;
    ewald2(chg, gstlentry[i], e2, m0);
    ewld2sum += e2;
    srfrce(sittyp, gstlentry[i], m0, ev);
    vdwsum += ev;
  }
  double ewld3sum = ewald3en[m0];
  estep = (-ewld1eng + ewld2sum + vdwsum - ewld3sum) / engunit;
  estep = estep - delrc / engunit;
  for (int i = 1; i <= maxmls; ++i) {
    int ik = loc2(m0, i);
    double d = delrc_mol[ik];
    if (i != m0) delE[i] -= (ewald1en[ik] + ewald2en[ik] + vdwen[ik] + d) / engunit;
  }
  delE[m0] -= estep;
  if (parts) {
    parts[0] = ewld1eng;
    parts[1] = ewld2sum;
    parts[2] = vdwsum;
  }
}

// cartesian (utility_pack.f:3695-3709)
void Sim::cartesian(double fa, double fb, double fc, double &x, double &y,
                    double &z) const {
  x = fa * cell[0] + fb * cell[3] + fc * cell[6];
  y = fa * cell[1] + fb * cell[4] + fc * cell[7];
  z = fa * cell[2] + fb * cell[5] + fc * cell[8];
}

// com (utility_pack.f:3565-3596)
void Sim::com(int natms, int molt, double &cx, double &cy, double &cz) const {
  cx = cy = cz = 0.0;
  double weight = 0.0;
  for (int i = 1; i <= natms; ++i) {
    double mass = mol[molt].wght[i];
    weight += mass;
    cx += newx[i] * mass;
    cy += newy[i] * mass;
    cz += newz[i] * mass;
  }
  cx /= weight;
  cy /= weight;
  cz /= weight;
}

// rotation (utility_pack.f:3480-3524): quaternion rotation about (cx,cy,cz).
void Sim::rotation(int natms, double cx, double cy, double cz, double q1,
                   double q2, double q3, double q4) {
  for (int i = 1; i <= natms; ++i) {
    newx[i] -= cx;
    newy[i] -= cy;
    newz[i] -= cz;
  }
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
  double tx[64], ty[64], tz[64];
  for (int i = 1; i <= natms; ++i) {
    tx[i] = Q[0] * newx[i] + Q[1] * newy[i] + Q[2] * newz[i];
    ty[i] = Q[3] * newx[i] + Q[4] * newy[i] + Q[5] * newz[i];
    tz[i] = Q[6] * newx[i] + Q[7] * newy[i] + Q[8] * newz[i];
  }
  for (int i = 1; i <= natms; ++i) {
    newx[i] = tx[i] + cx;
    newy[i] = ty[i] + cy;
    newz[i] = tz[i] + cz;
  }
}

// translate (utility_pack.f:3161-3218): shift, then wrap the centre of mass
// into the cell with floor().
void Sim::translate(int natms, int molt, double a, double b, double c) {
  for (int i = 1; i <= natms; ++i) {
    newx[i] = a + newx[i];
    newy[i] = b + newy[i];
    newz[i] = c + newz[i];
  }
  double cx, cy, cz;
  com(natms, molt, cx, cy, cz);
  double ssx = rcell[0] * cx + rcell[3] * cy + rcell[6] * cz;
  double ssy = rcell[1] * cx + rcell[4] * cy + rcell[7] * cz;
  double ssz = rcell[2] * cx + rcell[5] * cy + rcell[8] * cz;
  double xss = ssx - std::floor(ssx), yss = ssy - std::floor(ssy),
         zss = ssz - std::floor(ssz);
  double x = cell[0] * xss + cell[3] * yss + cell[6] * zss;
  double y = cell[1] * xss + cell[4] * yss + cell[7] * zss;
  double z = cell[2] * xss + cell[5] * yss + cell[8] * zss;
  double sx = x - cx, sy = y - cy, sz = z - cz;
  for (int i = 1; i <= natms; ++i) {
    newx[i] += sx;
    newy[i] += sy;
    newz[i] += sz;
  }
}

// random_ins (utility_pack.f:3220-3331)
void Sim::random_ins(int iguest) {
  double randa = rng.next(), randb = rng.next(), randc = rng.next();
  double rand1 = rng.next(), rand2 = rng.next(), rand3 = rng.next(),
         rand4 = rng.next();
  double xc, yc, zc;
  cartesian(randa, randb, randc, xc, yc, zc);
  int natms = mol[locguest[iguest]].natoms;
  for (int i = 1; i <= natms; ++i) {
    newx[i] = guestx[iguest][i];
    newy[i] = guesty[iguest][i];
    newz[i] = guestz[iguest][i];
  }
  double theta = rand1 * 2.0 * PI;
  double beta1 = 2.0 * rand2 - 1.0, beta2 = 2.0 * rand3 - 1.0,
         beta3 = 2.0 * rand4 - 1.0;
  double sintheta = std::sin(theta / 2.0);
  double norm = std::sqrt(beta1 * beta1 + beta2 * beta2 + beta3 * beta3);
  double u1 = beta1 / norm, u2 = beta2 / norm, u3 = beta3 / norm;
  double q1 = std::cos(theta / 2.0);
  double q2 = sintheta * u1, q3 = sintheta * u2, q4 = sintheta * u3;
  rotation(natms, 0.0, 0.0, 0.0, q1, q2, q3, q4);
  for (int i = 1; i <= natms; ++i) {
    newx[i] += xc;
    newy[i] += yc;
    newz[i] += zc;
  }
}

// random_disp (utility_pack.f:3333-3357)
void Sim::random_disp(double ddelr, double &a, double &b, double &c) {
  a = rng.next();
  b = rng.next();
  c = rng.next();
  double half = ddelr * 0.5;
  a = (2.0 * a - 1.0) * half;
  b = (2.0 * b - 1.0) * half;
  c = (2.0 * c - 1.0) * half;
}

// random_rot (utility_pack.f:3526-3563)
void Sim::random_rot(double rotang, double &q1, double &q2, double &q3,
                     double &q4) {
  double rand1 = rng.next(), rand2 = rng.next(), rand3 = rng.next(),
         rand4 = rng.next();
  double theta = rand1 * rotang;
  double beta1 = 2.0 * rand2 - 1.0, beta2 = 2.0 * rand3 - 1.0,
         beta3 = 2.0 * rand4 - 1.0;
  double sintheta = std::sin(theta / 2.0);
  double norm = std::sqrt(beta1 * beta1 + beta2 * beta2 + beta3 * beta3);
  double u1 = beta1 / norm, u2 = beta2 / norm, u3 = beta3 / norm;
  q1 = std::cos(theta / 2.0);
  q2 = sintheta * u1;
  q3 = sintheta * u2;
  q4 = sintheta * u3;
}

// displace_guest (gcmc.f:2816-2901)
void Sim::displace_guest(int iguest, int imol, double a, double b, double c,
                         double q1, double q2, double q3, double q4,
                         bool &linitsurf, bool &lnewsurf, bool &loverlap,
                         double &estep) {
  int m0, natms, nmols;
  get_guest(iguest, imol, m0, natms, nmols);
  int nmc = mxcmls();
  double vdwsum, ewld2sum, ewld1eng, chgtmp, engsictmp;
  guest_energy(iguest, vdwsum, ewld2sum, ewld1eng, linitsurf, chgtmp,
               engsictmp, loverlap, estep, true);
  double enginit = estep;
  for (int ik = 1; ik <= nmc; ++ik) {
    ewald1entmp[ik] = ewald1en[ik];
    ewald2entmp[ik] = ewald2en[ik];
    vdwentmp[ik] = vdwen[ik];
  }
  for (int ik = 1; ik <= newld; ++ik) {
    ckc(ckcsum, m0, ik) -= ckc(ckcsnew, m0, ik);
    ckc(ckssum, m0, ik) -= ckc(ckssnew, m0, ik);
    ckc(ckcsum, maxmls + 1, ik) -= ckc(ckcsnew, maxmls + 1, ik);
    ckc(ckssum, maxmls + 1, ik) -= ckc(ckssnew, maxmls + 1, ik);
  }
  translate(natms, m0, a, b, c);
  double cx, cy, cz;
  com(natms, m0, cx, cy, cz);
  rotation(natms, cx, cy, cz, q1, q2, q3, q4);
  guest_energy(iguest, vdwsum, ewld2sum, ewld1eng, lnewsurf, chgtmp, engsictmp,
               loverlap, estep, false);
  estep = estep - enginit;
  for (int i = 1; i <= maxmls; ++i) {
    int ik = loc2(m0, i);
    if (i != m0)
      delE[i] += (ewald1en[ik] - ewald1entmp[ik] + ewald2en[ik] - ewald2entmp[ik] +
                  vdwen[ik] - vdwentmp[ik]) /
                 engunit;
  }
  delE[m0] += estep;
}

// accept_move (mc_moves.f:485-621)
void Sim::accept_move(int iguest, bool insert, bool del, bool disp, bool lsurf,
                      double delrc, int &choice, double engsictmp,
                      double chgtmp) {
  int m0 = locguest[iguest];
  int kk = loc2(m0, m0);
  int natms = mol[m0].natoms;
  int at = (choice - 1) * natms + 1;
  int nmc = mxcmls();
  for (int i = 1; i <= maxmls; ++i) energy[i] += delE[i];
  MolType &m = mol[m0];
  if (insert) {
    for (int k = 1; k <= newld; ++k) {
      ckc(ckcsum, m0, k) += ckc(ckcsnew, m0, k);
      ckc(ckssum, m0, k) += ckc(ckssnew, m0, k);
      ckc(ckcsum, maxmls + 1, k) += ckc(ckcsnew, maxmls + 1, k);
      ckc(ckssum, maxmls + 1, k) += ckc(ckssnew, maxmls + 1, k);
    }
    engsic[kk] += engsictmp;
    chgsum_mol[m0] += chgtmp;
    sumchg += chgtmp;
    if (lsurf) surfacemols[m0] += 1;
    if (m.nummols + 1 > 20000) fail("oracle: maxguest exceeded");
    for (int i = 1; i <= natms; ++i) {
      m.mx.push_back(newx[i]);
      m.my.push_back(newy[i]);
      m.mz.push_back(newz[i]);
      int ka = m.ltp[i];
      numtyp[ka]++;
      numtyp_mol[m0][ka]++;
      if (m.frz[i] != 0) {
        numfrz[ka]++;
        numfrz_mol[m0][ka]++;
      }
    }
    elrc += delrc;
    for (int q = 1; q <= nmc; ++q) elrc_mol[q] += delrc_mol[q];
    m.nummols += 1;
    totatm += natms;
    condense();
    choice = m.nummols;
  } else if (del) {
    for (int k = 1; k <= newld; ++k) {
      ckc(ckcsum, m0, k) -= ckc(ckcsnew, m0, k);
      ckc(ckssum, m0, k) -= ckc(ckssnew, m0, k);
      ckc(ckcsum, maxmls + 1, k) -= ckc(ckcsnew, maxmls + 1, k);
      ckc(ckssum, maxmls + 1, k) -= ckc(ckssnew, maxmls + 1, k);
    }
    engsic[kk] -= engsictmp;
    chgsum_mol[m0] -= chgtmp;
    sumchg -= chgtmp;
    if (lsurf) surfacemols[m0] -= 1;
    for (int iatm = 1; iatm <= natms; ++iatm) {
      int ka = m.ltp[iatm];
      numtyp[ka]--;
      numtyp_mol[m0][ka]--;
      if (m.frz[iatm] != 0) {
        numfrz[ka]--;
        numfrz_mol[m0][ka]--;
      }
    }
    // shift the following molecules back (mc_moves.f:574-590)
    m.mx.erase(m.mx.begin() + at, m.mx.begin() + at + natms);
    m.my.erase(m.my.begin() + at, m.my.begin() + at + natms);
    m.mz.erase(m.mz.begin() + at, m.mz.begin() + at + natms);
    elrc -= delrc;
    for (int q = 1; q <= nmc; ++q) elrc_mol[q] -= delrc_mol[q];
    m.nummols -= 1;
    totatm -= natms;
    condense();
  } else if (disp) {
    for (int k = 1; k <= newld; ++k) {
      ckc(ckcsum, m0, k) += ckc(ckcsnew, m0, k);
      ckc(ckssum, m0, k) += ckc(ckssnew, m0, k);
      ckc(ckcsum, maxmls + 1, k) += ckc(ckcsnew, maxmls + 1, k);
      ckc(ckssum, maxmls + 1, k) += ckc(ckssnew, maxmls + 1, k);
    }
    int mm = 0;
    for (int i = at; i <= at - 1 + natms; ++i) {
      ++mm;
      m.mx[i] = newx[mm];
      m.my[i] = newy[mm];
      m.mz[i] = newz[mm];
    }
    condense();
  }
}

// reject_move (mc_moves.f:623-673)
void Sim::reject_move(int iguest, bool insert, bool del, bool disp) {
  (void)iguest;
  (void)disp;
  std::fill(delE.begin(), delE.end(), 0.0);
  if (insert || del) engsic = engsicorig;
}

// energy_eval (utility_pack.f:3637-3693)
bool Sim::energy_eval(double eng, double rande, int iguest, bool displace,
                      bool insert, bool del) {
  double test = 0.0;
  double ipress = gstfuga[iguest];
  int imol = locguest[iguest];
  int ingsts = mol[imol].nummols;
  double edummy = eng;
  if (-beta * edummy > 700.0)
    test = std::exp(700.0);
  else if (beta * edummy > 700.0)
    test = std::exp(-700.0);
  else if (displace)
    test = std::exp(-1.0 * beta * edummy);
  else if (insert)
    test = statvolm * ipress / ((double(ingsts) + 1.0) * BOLTZ * temp) *
           std::exp(-1.0 * beta * edummy);
  else if (del) {
    if (std::fabs(ipress) < 1.0e-7)
      test = 1.0;
    else
      test = double(ingsts) * BOLTZ * temp / (statvolm * ipress) *
             std::exp(-1.0 * beta * edummy);
  }
  return rande < test;
}

void fill_log_xyz(const Sim &S, int natms, orc_move_log *lg) {
  if (!lg) return;
  for (int i = 1; i <= natms && i <= 3; ++i) {
    lg->newxyz[3 * (i - 1) + 0] = S.newx[i];
    lg->newxyz[3 * (i - 1) + 1] = S.newy[i];
    lg->newxyz[3 * (i - 1) + 2] = S.newz[i];
  }
}

double sum_other_dele(const Sim &S, int m0) {
  double s = 0.0;
  for (int i = 1; i <= S.maxmls; ++i)
    if (i != m0) s += S.delE[i];
  return s;
}

// mc_insert (gcmc.f:1693-1752)
void Sim::mc_insert(int iguest, orc_move_log *lg) {
  int m0 = locguest[iguest];
  bool lnewsurf = false, loverlap = false;
  engsicorig = engsic;
  ins_count[iguest]++;
  random_ins(iguest);
  double estep = 0.0, delrc = 0.0, chgtmp = 0.0, engsictmp = 0.0;
  insertion(iguest, delrc, estep, chgtmp, engsictmp, loverlap, lnewsurf, nullptr);
  bool accepted = false;
  double rande = -1.0;
  if (!loverlap) {
    rande = rng.next();
    accepted = energy_eval(estep, rande, iguest, false, true, false);
  }
  fill_log_xyz(*this, mol[m0].natoms, lg);
  if (lg) {
    lg->move = 1;
    lg->choice = 0;
    lg->overlap = loverlap;
    lg->estep = estep;
    lg->rande = rande;
    lg->dele_other = sum_other_dele(*this, m0);
  }
  if (accepted) {
    accept_ins[iguest]++;
    int rc = 0;
    accept_move(iguest, true, false, false, lnewsurf, delrc, rc, engsictmp, chgtmp);
  } else {
    reject_move(iguest, true, false, false);
  }
  production_stats(accepted);
  if (lg) lg->accepted = accepted;
}

// mc_delete (gcmc.f:1754-1810)
void Sim::mc_delete(int iguest, orc_move_log *lg) {
  int m0 = locguest[iguest];
  int nmol = mol[m0].nummols;
  engsicorig = engsic;
  bool linitsurf = false;
  del_count[iguest]++;
  int randchoice = (int)std::floor(rng.next() * nmol) + 1;
  double estep = 0.0, delrc = 0.0, engsictmp = 0.0, chgtmp = 0.0;
  deletion(iguest, randchoice, delrc, estep, linitsurf, engsictmp, chgtmp, nullptr);
  double rande = rng.next();
  bool accepted = energy_eval(-estep, rande, iguest, false, false, true);
  fill_log_xyz(*this, mol[m0].natoms, lg);
  if (lg) {
    lg->move = 2;
    lg->choice = randchoice;
    lg->overlap = 0;
    lg->estep = estep;
    lg->rande = rande;
    lg->dele_other = sum_other_dele(*this, m0);
  }
  if (accepted) {
    accept_del[iguest]++;
    accept_move(iguest, false, true, false, linitsurf, delrc, randchoice,
                engsictmp, chgtmp);
  } else {
    reject_move(iguest, false, true, false);
  }
  production_stats(accepted);
  if (lg) lg->accepted = accepted;
}

// mc_displace (gcmc.f:1812-1935)
void Sim::mc_displace(int iguest, bool tran, bool rota, orc_move_log *lg) {
  int m0 = locguest[iguest];
  int nmol = mol[m0].nummols;
  double a = 0, b = 0, c = 0, q1 = 0, q2 = 0, q3 = 0, q4 = 0;
  if (tran) {
    tran_count[iguest]++;
    random_disp(tran_delr[iguest], a, b, c);
  } else if (rota) {
    rota_count[iguest]++;
    random_rot(rota_rotangle, q1, q2, q3, q4);
  } else {
    disp_count[iguest]++;
    random_disp(delrdisp[iguest], a, b, c);
    random_rot(rotangle, q1, q2, q3, q4);
  }
  for (int ik = 1; ik <= newld; ++ik) {
    ckc(ckcsorig, m0, ik) = ckc(ckcsum, m0, ik);
    ckc(ckssorig, m0, ik) = ckc(ckssum, m0, ik);
    ckc(ckcsorig, maxmls + 1, ik) = ckc(ckcsum, maxmls + 1, ik);
    ckc(ckssorig, maxmls + 1, ik) = ckc(ckssum, maxmls + 1, ik);
  }
  int randchoice = (int)std::floor(rng.next() * nmol) + 1;
  bool linitsurf = false, lnewsurf = false, loverlap = false;
  double estep = 0.0;
  displace_guest(iguest, randchoice, a, b, c, q1, q2, q3, q4, linitsurf,
                 lnewsurf, loverlap, estep);
  bool accepted = false;
  double rande = -1.0;
  if (!loverlap) {
    if (estep < 0.0) {
      accepted = true;
    } else {
      rande = rng.next();
      accepted = energy_eval(estep, rande, iguest, true, false, false);
    }
  }
  fill_log_xyz(*this, mol[m0].natoms, lg);
  if (lg) {
    lg->move = tran ? 4 : (rota ? 5 : 3);
    lg->choice = randchoice;
    lg->overlap = loverlap;
    lg->estep = estep;
    lg->rande = rande;
    lg->dele_other = sum_other_dele(*this, m0);
  }
  if (accepted) {
    int rc = randchoice;
    accept_move(iguest, false, false, true, lnewsurf, 0.0, rc, 0.0, 0.0);
    if (linitsurf && !lnewsurf) {
      surfacemols[m0] -= 1;
      if (surfacemols[m0] < 0) surfacemols[m0] = 0;
    } else if (!linitsurf && lnewsurf) {
      surfacemols[m0] += 1;
    }
    if (tran)
      accept_tran[iguest]++;
    else if (rota)
      accept_rota[iguest]++;
    else
      accept_disp[iguest]++;
  } else {
    for (int ik = 1; ik <= newld; ++ik) {
      ckc(ckcsum, m0, ik) = ckc(ckcsorig, m0, ik);
      ckc(ckssum, m0, ik) = ckc(ckssorig, m0, ik);
      ckc(ckcsum, maxmls + 1, ik) = ckc(ckcsorig, maxmls + 1, ik);
      ckc(ckssum, maxmls + 1, ik) = ckc(ckssorig, maxmls + 1, ik);
    }
    reject_move(iguest, false, false, true);
  }
  production_stats(accepted);
  if (lg) lg->accepted = accepted;
}

// mc_jump (gcmc.f:1937-2039): a random molecule moved to a random point of
// the cell (random_jump, utility_pack.f:3359-3380) with a random
// orientation (random_rot with angle 2 pi), written as the translation
// a,b,c = new centre - old centre of mass for displace_guest.
void Sim::mc_jump(int iguest, orc_move_log *lg) {
  int m0 = locguest[iguest];
  int nmol = mol[m0].nummols;
  int natms = mol[m0].natoms;
  jump_count[iguest]++;
  int randchoice = (int)std::floor(rng.next() * nmol) + 1;
  for (int ik = 1; ik <= newld; ++ik) {
    ckc(ckcsorig, m0, ik) = ckc(ckcsum, m0, ik);
    ckc(ckssorig, m0, ik) = ckc(ckssum, m0, ik);
    ckc(ckcsorig, maxmls + 1, ik) = ckc(ckcsum, maxmls + 1, ik);
    ckc(ckssorig, maxmls + 1, ik) = ckc(ckssum, maxmls + 1, ik);
  }
  int molt = 0, na = 0, nm = 0;
  get_guest(iguest, randchoice, molt, na, nm);
  double comx, comy, comz;
  com(natms, m0, comx, comy, comz);
  double randa = rng.next(), randb = rng.next(), randc = rng.next();  // random_jump
  double xc, yc, zc;
  cartesian(randa, randb, randc, xc, yc, zc);
  const double jumpangle = 8.0 * std::atan(1.0);
  double q1, q2, q3, q4;
  random_rot(jumpangle, q1, q2, q3, q4);
  const double a = xc - comx, b = yc - comy, c = zc - comz;
  bool linitsurf = false, lnewsurf = false, loverlap = false;
  double estep = 0.0;
  displace_guest(iguest, randchoice, a, b, c, q1, q2, q3, q4, linitsurf, lnewsurf, loverlap, estep);
  bool accepted = false;
  double rande = -1.0;
  if (!loverlap) {
    if (estep < 0.0) {
      accepted = true;
    } else {
      rande = rng.next();
      accepted = energy_eval(estep, rande, iguest, true, false, false);
    }
  }
  fill_log_xyz(*this, natms, lg);
  if (lg) {
    lg->move = 6;
    lg->choice = randchoice;
    lg->overlap = loverlap;
    lg->estep = estep;
    lg->rande = rande;
    lg->dele_other = sum_other_dele(*this, m0);
  }
  if (accepted) {
    accept_jump[iguest]++;
    int rc = randchoice;
    accept_move(iguest, false, false, true, lnewsurf, 0.0, rc, 0.0, 0.0);
    if (linitsurf && !lnewsurf) {
      surfacemols[m0] -= 1;
      if (surfacemols[m0] < 0) surfacemols[m0] = 0;
    } else if (!linitsurf && lnewsurf) {
      surfacemols[m0] += 1;
    }
  } else {
    for (int ik = 1; ik <= newld; ++ik) {
      ckc(ckcsum, m0, ik) = ckc(ckcsorig, m0, ik);
      ckc(ckssum, m0, ik) = ckc(ckssorig, m0, ik);
      ckc(ckcsum, maxmls + 1, ik) = ckc(ckcsorig, maxmls + 1, ik);
      ckc(ckssum, maxmls + 1, ik) = ckc(ckssorig, maxmls + 1, ik);
    }
    reject_move(iguest, false, false, true);
  }
  production_stats(accepted);
  if (lg) lg->accepted = accepted;
}

double calc_qst(double E, double N, double N2, double EN, double temp) {
  double q = 0.0, denom = N2 - N * N;
  if (std::fabs(denom) > 0.0) q = -1.0 * (EN - E * N) / denom + RGAS * temp;
  return q;
}
double calc_cv(double E2, double E, double N, double N2, double EN, double temp) {
  double cv = 0.0, denom = N2 - N * N;
  if (std::fabs(denom) > 0.0 && N > 0.0)
    cv = (3.0 / 2.0 * RGAS) + (E2 - (E * E) - (EN - E * N) * (EN - E * N) / denom) /
                                  (N * KBOLTZ * temp * temp);
  return cv;
}

// production statistics (gcmc.f:1050-1128)
// mc_swap (gcmc.f:2269-2452) after its draws: molecule `ichoice` of
// iguest is deleted and committed, a molecule of jguest is built from its
// template at the deleted centre of mass, rotated by q, inserted and
// committed, and the pair is accepted when rande[0] < testi and then
// rande[1] < testj.  A rejection restores what the reference saves:
// coordinates and S(k) of both types, their chgsum_mol and surfacemols,
// elrc, totatm, the counts and energy(); reject_move's swap branch
// (mc_moves.f:646-669) restores engsic, elrc_mol and the site-type counts.
// sumchg keeps the two accept_move updates (the reference does not save it).
// out (if given): estepi, estepj, loverlap, accepted.
void Sim::swap_move(int iguest, int ichoice, int jguest, const double *q,
                    const double *rande, double *out, orc_move_log *lg) {
  const int imol = locguest[iguest], jmol = locguest[jguest];
  swap_count[iguest]++;
  std::vector<double> origenergy = energy;
  const double ochg_i = chgsum_mol[imol], ochg_j = chgsum_mol[jmol];
  const double osurf_i = surfacemols[imol], osurf_j = surfacemols[jmol];
  engsicorig = engsic;
  origelrc = elrc;
  origelrc_mol = elrc_mol;
  const int origtotatm = totatm;
  const std::vector<double> oix = mol[imol].mx, oiy = mol[imol].my, oiz = mol[imol].mz;
  const std::vector<double> ojx = mol[jmol].mx, ojy = mol[jmol].my, ojz = mol[jmol].mz;
  const std::vector<double> ockc = ckcsum, ocks = ckssum;
  int molt, natms, nm;
  get_guest(iguest, ichoice, molt, natms, nm);
  double cx, cy, cz;
  com(natms, imol, cx, cy, cz);
  // delete the first guest and commit
  double estep = 0.0, delrc = 0.0, engsictmp = 0.0, chgtmp = 0.0;
  bool linitsurf = false;
  deletion(iguest, ichoice, delrc, estep, linitsurf, engsictmp, chgtmp, nullptr);
  int ch = ichoice;
  accept_move(iguest, false, true, false, linitsurf, delrc, ch, engsictmp, chgtmp);
  const double estepi = -estep;
  // insert the second guest at the centre of mass and commit
  const int jn = mol[jmol].natoms;
  for (int i = 1; i <= jn; ++i) {
    newx[i] = guestx[jguest][i] + cx;
    newy[i] = guesty[jguest][i] + cy;
    newz[i] = guestz[jguest][i] + cz;
  }
  rotation(jn, cx, cy, cz, q[0], q[1], q[2], q[3]);
  fill_log_xyz(*this, jn, lg);
  estep = delrc = chgtmp = engsictmp = 0.0;
  bool loverlap = false, lnewsurf = false;
  insertion(jguest, delrc, estep, chgtmp, engsictmp, loverlap, lnewsurf, nullptr);
  int jc = 0;
  accept_move(jguest, true, false, false, lnewsurf, delrc, jc, engsictmp, chgtmp);
  const double estepj = estep;
  bool accepted = false;
  double r0 = -1.0;
  if (!loverlap) {
    r0 = rande ? rande[0] : rng.next();
    const double jpress = gstfuga[jguest], ipress = gstfuga[iguest];
    const int jnmols = mol[jmol].nummols;
    const int inmols = mol[imol].nummols + 1;
    const double testi = double(inmols) * BOLTZ * temp / (volm * ipress) *
                         std::exp(-1.0 * beta * estepi);
    const double testj = volm * jpress / (double(jnmols) * BOLTZ * temp) *
                         std::exp(-1.0 * beta * estepj);
    if (r0 < testi) {
      const double r1 = rande ? rande[1] : rng.next();
      if (r1 < testj) accepted = true;
    }
  }
  if (accepted) {
    accept_swap[iguest]++;
    condense();
  } else {
    // reject_move(iguest, jguest, swap) (mc_moves.f:634-669)
    std::fill(delE.begin(), delE.end(), 0.0);
    engsic = engsicorig;
    elrc_mol = origelrc_mol;
    const MolType &mi = mol[imol], &mj = mol[jmol];
    for (int i = 1; i <= mi.natoms; ++i) {
      int ka = mi.ltp[i];
      numtyp[ka]++;
      numtyp_mol[imol][ka]++;
      if (mi.frz[i] != 0) {
        numfrz[ka]++;
        numfrz_mol[imol][ka]++;
      }
    }
    for (int i = 1; i <= mj.natoms; ++i) {
      int ka = mj.ltp[i];
      numtyp[ka]--;
      numtyp_mol[jmol][ka]--;
      if (mj.frz[i] != 0) {
        numfrz[ka]--;
        numfrz_mol[jmol][ka]--;
      }
    }
    mol[imol].mx = oix;
    mol[imol].my = oiy;
    mol[imol].mz = oiz;
    mol[jmol].mx = ojx;
    mol[jmol].my = ojy;
    mol[jmol].mz = ojz;
    ckcsum = ockc;
    ckssum = ocks;
    chgsum_mol[imol] = ochg_i;
    chgsum_mol[jmol] = ochg_j;
    surfacemols[imol] = osurf_i;
    surfacemols[jmol] = osurf_j;
    elrc = origelrc;
    totatm = origtotatm;
    mol[imol].nummols += 1;
    mol[jmol].nummols -= 1;
    condense();
    energy = origenergy;
  }
  if (lg) {
    lg->move = 7;
    lg->choice = ichoice;
    lg->overlap = loverlap;
    lg->accepted = accepted;
    lg->estep = estepi + estepj;
    lg->rande = r0;
  }
  if (out) {
    out[0] = estepi;
    out[1] = estepj;
    out[2] = loverlap ? 1.0 : 0.0;
    out[3] = accepted ? 1.0 : 0.0;
  }
  production_stats(accepted);
}

// mc_switch (gcmc.f:2041-2267).  With fewer than two other guest types
// holding molecules it returns before any draw, and the main loop's
// `accepted` keeps the previous move's value.  Otherwise a molecule of
// iguest and one of a partner type exchange centres of mass, each keeping
// its orientation: both are deleted and committed, then the partner is
// inserted at the first's centre and the first at the partner's, each
// committed even when it overlaps; the pair is accepted when the summed
// change is negative, else by energy_eval's displacement test (drawn
// before the overlap veto).  A rejection restores energy(), surfacemols,
// coordinates and S(k) of both types and engsic, and sets elrc and
// elrc_mol to mc_swap's saved values (zero before any swap).
void Sim::mc_switch(int iguest, orc_move_log *lg) {
  std::vector<int> chosen(1, 0);  // switch_chosen_guest, 1-based
  for (int i = 1; i <= ntpguest; ++i)
    if (mol[locguest[i]].nummols > 0 && i != iguest) chosen.push_back(i);
  const int nswitchgst = (int)chosen.size() - 1;
  if (nswitchgst < 2) {
    if (lg) {
      lg->move = 0;
      lg->accepted = last_accepted;
    }
    production_stats(last_accepted);
    return;
  }
  switch_count[iguest]++;
  engsicorig = engsic;
  bool loverallap = false;
  const int jguest = chosen[(int)std::floor(rng.next() * nswitchgst) + 1];
  const int imol = locguest[iguest], jmol = locguest[jguest];
  const int ichoice = (int)std::floor(rng.next() * mol[imol].nummols) + 1;
  const int jchoice = (int)std::floor(rng.next() * mol[jmol].nummols) + 1;
  const std::vector<double> origenergy = energy, origsurf = surfacemols;
  const std::vector<double> oix = mol[imol].mx, oiy = mol[imol].my, oiz = mol[imol].mz;
  const std::vector<double> ojx = mol[jmol].mx, ojy = mol[jmol].my, ojz = mol[jmol].mz;
  const std::vector<double> ockc = ckcsum, ocks = ckssum;
  // both molecules' orientations about their centres of mass
  int molt, jn, in, nm;
  double jc[3], ic[3];
  get_guest(jguest, jchoice, molt, jn, nm);
  com(jn, jmol, jc[0], jc[1], jc[2]);
  std::vector<double> gj(3 * jn + 3);
  for (int a = 1; a <= jn; ++a) {
    gj[3 * a] = newx[a] - jc[0];
    gj[3 * a + 1] = newy[a] - jc[1];
    gj[3 * a + 2] = newz[a] - jc[2];
  }
  get_guest(iguest, ichoice, molt, in, nm);
  com(in, imol, ic[0], ic[1], ic[2]);
  std::vector<double> gi(3 * in + 3);
  for (int a = 1; a <= in; ++a) {
    gi[3 * a] = newx[a] - ic[0];
    gi[3 * a + 1] = newy[a] - ic[1];
    gi[3 * a + 2] = newz[a] - ic[2];
  }
  // delete both and commit
  double estep = 0.0, delrc = 0.0, engsictmp = 0.0, chgtmp = 0.0;
  bool linitsurf = false, linitsurfj = false;
  deletion(iguest, ichoice, delrc, estep, linitsurf, engsictmp, chgtmp, nullptr);
  int ch = ichoice;
  accept_move(iguest, false, true, false, linitsurf, delrc, ch, engsictmp, chgtmp);
  double estepi = -estep;
  estep = 0.0;
  deletion(jguest, jchoice, delrc, estep, linitsurfj, engsictmp, chgtmp, nullptr);
  ch = jchoice;
  accept_move(jguest, false, true, false, linitsurfj, delrc, ch, engsictmp, chgtmp);
  double estepj = -estep;
  // the partner at the first molecule's centre, then the first at the
  // partner's, each committed
  for (int a = 1; a <= jn; ++a) {
    newx[a] = gj[3 * a] + ic[0];
    newy[a] = gj[3 * a + 1] + ic[1];
    newz[a] = gj[3 * a + 2] + ic[2];
  }
  estep = 0.0;
  bool loverlap = false, lnewsurfj = false, lnewsurf = false;
  insertion(jguest, delrc, estep, chgtmp, engsictmp, loverlap, lnewsurfj, nullptr);
  if (loverlap) loverallap = true;
  estepj += estep;
  ch = jchoice;
  accept_move(jguest, true, false, false, lnewsurfj, delrc, ch, engsictmp, chgtmp);
  for (int a = 1; a <= in; ++a) {
    newx[a] = gi[3 * a] + jc[0];
    newy[a] = gi[3 * a + 1] + jc[1];
    newz[a] = gi[3 * a + 2] + jc[2];
  }
  fill_log_xyz(*this, in, lg);
  estep = 0.0;
  insertion(iguest, delrc, estep, chgtmp, engsictmp, loverlap, lnewsurf, nullptr);
  if (loverlap) loverallap = true;
  estepi += estep;
  ch = ichoice;
  accept_move(iguest, true, false, false, lnewsurf, delrc, ch, engsictmp, chgtmp);
  bool accepted;
  double rande = -1.0;
  if (estepi + estepj < 0.0) {
    accepted = true;
  } else {
    rande = rng.next();
    accepted = energy_eval(estepi + estepj, rande, iguest, true, false, false);
  }
  if (loverallap) accepted = false;
  if (accepted) {
    accept_switch[iguest]++;
    condense();
  } else {
    for (int ik = 1; ik <= maxmls; ++ik) {
      delE[ik] = 0.0;
      energy[ik] = origenergy[ik];
      surfacemols[ik] = origsurf[ik];
    }
    mol[imol].mx = oix;
    mol[imol].my = oiy;
    mol[imol].mz = oiz;
    mol[jmol].mx = ojx;
    mol[jmol].my = ojy;
    mol[jmol].mz = ojz;
    ckcsum = ockc;
    ckssum = ocks;
    elrc = origelrc;
    if (origelrc_mol.empty()) origelrc_mol.assign(elrc_mol.size(), 0.0);
    elrc_mol = origelrc_mol;
    engsic = engsicorig;
    condense();
  }
  if (lg) {
    lg->move = 8;
    lg->choice = ichoice;
    lg->overlap = loverallap;
    lg->accepted = accepted;
    lg->estep = estepi + estepj;
    lg->rande = rande;
  }
  production_stats(accepted);
}

// mc_swap's draws (gcmc.f:2313-2318, 2349): the molecule, the partner
// type among the others (switch_chosen_guest), and random_rot's quaternion
// with the displacement angle
void Sim::mc_swap(int iguest, orc_move_log *lg) {
  if (ntpguest < 2) fail("oracle: swap moves need two guest types");
  const int nmols = mol[locguest[iguest]].nummols;
  const int ichoice = (int)std::floor(rng.next() * nmols + 1);
  int jg = (int)std::floor(rng.next() * (ntpguest - 1) + 1);
  const int jguest = jg < iguest ? jg : jg + 1;
  double q[4];
  random_rot(rotangle, q[0], q[1], q[2], q[3]);
  swap_move(iguest, ichoice, jguest, q, nullptr, nullptr, lg);
}

void Sim::production_stats(bool accepted) {
  last_accepted = accepted;
  if (!production) return;
  if (lprob) storeprob();  // gcmc.f:1129-1130, every production move
  // gcmc.f:1131-1134: storeenprob(iguest, randchoice, ..., guest_toten) with
  // the main program's randchoice and guest_toten, which no routine sets
  // (the move routines' variables of those names are their own): molecule
  // 0, so newx as the move left it, and energy 0
  if (lprob && lprobeng[cur_iguest] && accepted) storeenprob(cur_iguest, 0.0);
  if (!((laccsample && accepted) || !laccsample)) return;
  ++prodcount;
  ++rollcount;
  chainstats[1] = double(prodcount);
  for (int i = 1; i <= ntpguest; ++i) {
    int m = locguest[i];
    double dm = double((float)mol[m].nummols);
    double e = energy[m];
    double sm = double((float)surfacemols[m]);
    int is = 1 + 16 * (i - 1);
    chainstats[is + 1] += dm;
    chainstats[is + 2] += e;
    chainstats[is + 3] += e * dm;
    chainstats[is + 4] += dm * dm;
    chainstats[is + 5] += e * e;
    chainstats[is + 6] += sm;
  }
  long long testcount = prodcount;
  if (testcount % nwindsteps == 0) {
    std::vector<double> w(1 + 9 * ntpguest + 1, 0.0);
    w[1] = double(rollcount);
    for (int i = 1; i <= ntpguest; ++i) {
      int is = 1 + (i - 1) * 16, rs = 1 + (i - 1) * 9;
      double rc = double(rollcount);
      double aN = chainstats[is + 1] / rc, E = chainstats[is + 2] / rc,
             EN = chainstats[is + 3] / rc, N2 = chainstats[is + 4] / rc,
             E2 = chainstats[is + 5] / rc, NF = chainstats[is + 6] / rc;
      w[rs + 1] = aN;
      w[rs + 2] = E;
      w[rs + 3] = EN;
      w[rs + 4] = N2;
      w[rs + 5] = E2;
      w[rs + 6] = NF;
      w[rs + 7] = calc_qst(E, aN, N2, EN, temp);
      w[rs + 8] = calc_cv(E2, E, aN, N2, EN, temp);
      for (int q = 1; q <= 6; ++q) chainstats[is + q] = 0.0;
    }
    avgwindow.push_back(w);
    rollcount = 0;
  }
}

// Grid dimensions and the folding cell (gcmc.f:258-306): voxels of about
// griddim per unit-cell edge, the unit cell = cell / gridfactor per vector.
void Sim::setup_grid() {
  for (int i = 1; i <= 9; ++i) {
    int ci = (int)std::ceil(double(i) / 3.0);
    ucell[i - 1] = cell[i - 1] / double(gridfactor[ci - 1]);
  }
  double det;
  invert(ucell, rucell, det);
  if (!lprob) return;
  double gd[3];
  int ng[3];
  for (int d = 0; d < 3; ++d) {
    gd[d] = celprp[d] / std::ceil(celprp[d] / gridfactor[d] / griddim) / gridfactor[d];
    ng[d] = (int)std::ceil(celprp[d] / (gd[d] * gridfactor[d]));
  }
  ngrida = ng[0];
  ngridb = ng[1];
  ngridc = ng[2];
  gridsize = ngrida * ngridb * ngridc;
  grid.assign((size_t)std::max(ntprob, 1) * gridsize, 0.0);
}

// equitable_bin (utility_pack.f:2407-2519): val spread over the 2x2x2 voxels
// around a fractional point, weights linear in the distance to the voxel
// centres; the periodic wraps (including the b-direction offset of 1 at the
// upper edge) as the reference has them.
void Sim::equitable_bin(double fa, double fb, double fc, int sub, double val) {
  const int na = ngrida, nb = ngridb, nc = ngridc;
  int alidx, aridx, blidx, bridx, clidx, cridx;
  double al, ar, bl, br, cl, cr;
  double gpta = na * fa;
  int aidx = (int)std::ceil(gpta);
  double apart = gpta - std::floor(gpta);  // modulo(gpta, 1.d0)
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
  double gptb = nb * fb;
  int bidx = (int)std::ceil(gptb);
  double bpart = gptb - std::floor(gptb);
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
  double gptc = nc * fc;
  int cidx = (int)std::ceil(gptc);
  double cpart = gptc - std::floor(gptc);
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
  double *g = grid.data() + (size_t)(sub - 1) * gridsize - 1;  // bins are 1-based
  g[alidx + blidx + clidx] += (al * bl * cl) * val;
  g[aridx + blidx + clidx] += (ar * bl * cl) * val;
  g[alidx + bridx + clidx] += (al * br * cl) * val;
  g[alidx + blidx + cridx] += (al * bl * cr) * val;
  g[aridx + bridx + clidx] += (ar * br * cl) * val;
  g[aridx + blidx + cridx] += (ar * bl * cr) * val;
  g[alidx + bridx + cridx] += (al * br * cr) * val;
  g[aridx + bridx + cridx] += (ar * br * cr) * val;
}

// storeprob (utility_pack.f:621-687): every guest molecule's centre of mass
// or listed sites, folded into the unit cell, binned with weight 1.
void Sim::storeprob() {
  int itprob = 0;
  for (int ig = 1; ig <= ntpguest; ++ig) {
    int np = nprob[ig];
    if (lprobeng[ig]) np -= 2;
    int m0 = locguest[ig];
    int nmols = mol[m0].nummols, natms = mol[m0].natoms;
    int jj = 0;
    for (int im = 1; im <= nmols; ++im) {
      double x[kMaxProbSites + 1], y[kMaxProbSites + 1], z[kMaxProbSites + 1];
      if (natms > kMaxProbSites) fail("oracle: guest too large for storeprob");
      for (int a = 1; a <= natms; ++a) {
        ++jj;
        x[a] = mol[m0].mx[jj];
        y[a] = mol[m0].my[jj];
        z[a] = mol[m0].mz[jj];
      }
      double cx = 0, cy = 0, cz = 0, w = 0;
      for (int a = 1; a <= natms; ++a) {  // com (utility_pack.f:3565-3598)
        double mass = mol[m0].wght[a];
        w += mass;
        cx += x[a] * mass;
        cy += y[a] * mass;
        cz += z[a] * mass;
      }
      cx /= w;
      cy /= w;
      cz /= w;
      auto fold = [&](double &px, double &py, double &pz) {  // frac2 / frac
        const double *rc = rucell;
        double sx = px * rc[0] + py * rc[3] + pz * rc[6];
        double sy = px * rc[1] + py * rc[4] + pz * rc[7];
        double sz = px * rc[2] + py * rc[5] + pz * rc[8];
        px = sx - std::floor(sx);
        py = sy - std::floor(sy);
        pz = sz - std::floor(sz);
      };
      fold(cx, cy, cz);
      for (int a = 1; a <= natms; ++a) fold(x[a], y[a], z[a]);
      for (int ip = 1; ip <= np; ++ip) {
        int sub = itprob + ip;
        for (int i = 1; i <= nprobsites[sub]; ++i) {
          int jatm = lprobsites[sub][i];
          if (jatm == 0) equitable_bin(cx, cy, cz, sub, 1.0);
          else equitable_bin(x[jatm], y[jatm], z[jatm], sub, 1.0);
        }
      }
    }
    itprob += np;
    if (lprobeng[ig]) itprob += 2;
  }
}

// storeenprob (utility_pack.f:550-618) with imol 0: the centre of mass of
// newx (the guest type's site count and masses), folded into the unit cell,
// binned into the guest type's last two grids: the energy into the first,
// a count into the second.
void Sim::storeenprob(int iguest, double energy) {
  const int m0 = locguest[iguest];
  double cx, cy, cz;
  com(mol[m0].natoms, m0, cx, cy, cz);
  const double *rc = rucell;  // frac2
  const double sx = cx * rc[0] + cy * rc[3] + cz * rc[6];
  const double sy = cx * rc[1] + cy * rc[4] + cz * rc[7];
  const double sz = cx * rc[2] + cy * rc[5] + cz * rc[8];
  cx = sx - std::floor(sx);
  cy = sy - std::floor(sy);
  cz = sz - std::floor(sz);
  int itprob = 0;
  for (int j = 1; j <= ntpguest; ++j) {
    itprob += nprob[j];
    if (j == iguest) break;
  }
  equitable_bin(cx, cy, cz, itprob - 1, energy);
  equitable_bin(cx, cy, cz, itprob, 1.0);
}

// One iteration of the main loop (gcmc.f:704-1164), moves ins/del/dis/tra/rot.
void Sim::step(orc_move_log *lg) {
  ++cycle_step;
  ++gcmccount;
  if (gcmccount % minchk == 0) {
    if (!production && eqsteps > 0 && gcmccount >= eqsteps) production = true;
  }
  int iguest = 1;
  if (ntpguest > 1) iguest = (int)std::floor(rng.next() * ntpguest) + 1;
  int m0 = locguest[iguest];
  int nmols = mol[m0].nummols;
  double randmov = rng.next();
  bool insert = false, del = false, disp = false, tran = false, rota = false, jump = false,
       sw = false, swp = false;
  if (randmov < mcinsf[iguest]) insert = true;
  else if (randmov < mcdelf[iguest]) del = true;
  else if (randmov < mcdisf[iguest]) disp = true;
  else if (randmov < mcjmpf[iguest]) jump = true;
  else if (randmov < mcswpf[iguest]) swp = true;
  else if (randmov < mctraf[iguest]) { disp = true; tran = true; }
  else if (randmov < mcrotf[iguest]) { disp = true; rota = true; }
  else if (randmov < mcswif[iguest]) sw = true;
  else disp = true;
  // adaptive step sizes (gcmc.f:859-900)
  if (nmols >= 1 && disp_count[iguest] >= 1) {
    double ratio = double(accept_disp[iguest]) / double(disp_count[iguest]);
    if (disp_count[iguest] % 100 == 0) {
      if (ratio > disp_ratio[iguest])
        delrdisp[iguest] *= 1.05;
      else if (delrdisp[iguest] > DELRMIN)
        delrdisp[iguest] *= 0.95;
    } else if (disp_count[iguest] % 50 == 0) {
      if (ratio > disp_ratio[iguest])
        rotangle *= 1.05;
      else if (rotangle > MINANGLE)
        rotangle *= 0.95;
    }
  }
  if (nmols >= 1 && tran_count[iguest] >= 1 && tran_count[iguest] % 100 == 0) {
    double ratio = double(accept_tran[iguest]) / double(tran_count[iguest]);
    if (ratio > tran_ratio[iguest])
      tran_delr[iguest] *= 1.05;
    else if (tran_delr[iguest] > DELRMIN)
      tran_delr[iguest] *= 0.95;
  }
  if (nmols >= 1 && rota_count[iguest] >= 1 && rota_count[iguest] % 100 == 0) {
    double ratio = double(accept_rota[iguest]) / double(rota_count[iguest]);
    if (ratio > rota_ratio[iguest])
      rota_rotangle *= 1.05;
    else if (rota_rotangle > MINANGLE)
      rota_rotangle *= 0.95;
  }
  if (nmols == 0) {
    insert = true;
    del = disp = tran = rota = jump = sw = swp = false;
  }
  if (lg) {
    std::memset(lg, 0, sizeof(*lg));
    lg->iguest = iguest;
  }
  cur_iguest = iguest;
  if (insert) {
    mc_insert(iguest, lg);
  } else if (del) {
    mc_delete(iguest, lg);
  } else if (jump) {
    mc_jump(iguest, lg);
  } else if (swp) {
    mc_swap(iguest, lg);
  } else if (sw) {
    mc_switch(iguest, lg);
  } else {
    mc_displace(iguest, tran, rota, lg);
  }
  if (lg) lg->nmols_after = mol[m0].nummols;
}

// True when a trial position (newx/newy/newz, sites 1..natms) lies within
// the overlap distance of a framework atom by a clear margin, with the
// distance formed as insertion() forms it (difference, images, sum of
// squares).  Such a trial is rejected by insertion() whatever else it
// finds, and its rejection leaves no state behind, so insert_guests may
// skip the call.  Orthorhombic cells only (false otherwise); trials near
// the threshold or overlapping only guests still go through insertion().
bool Sim::fw_overlap_certain(int natms) {
  if (imcon != 1 && imcon != 2) return false;
  const double L[3] = {cell[0], cell[4], cell[8]};
  const double ovd = std::sqrt(overlap);
  if (!fwgrid.built) {
    fwgrid.built = true;
    for (int d = 0; d < 3; ++d) {
      fwgrid.nc[d] = std::max(3, (int)std::floor(L[d] / std::max(ovd, 1e-3)));
      fwgrid.csz[d] = L[d] / fwgrid.nc[d];
    }
    const int ncell = fwgrid.nc[0] * fwgrid.nc[1] * fwgrid.nc[2];
    std::vector<std::vector<double>> bx(ncell), by(ncell), bz(ncell);
    for (int fr = 1; fr <= ntpfram; ++fr) {
      const MolType &m = mol[locfram[fr]];
      const int n = m.nummols * m.natoms;
      for (int i = 1; i <= n; ++i) {
        const double p[3] = {m.mx[i], m.my[i], m.mz[i]};
        int c3[3];
        for (int d = 0; d < 3; ++d) {
          const double w = p[d] - L[d] * std::floor(p[d] / L[d]);
          c3[d] = std::min(fwgrid.nc[d] - 1, std::max(0, (int)(w / fwgrid.csz[d])));
        }
        const int c = (c3[0] * fwgrid.nc[1] + c3[1]) * fwgrid.nc[2] + c3[2];
        bx[c].push_back(p[0]);
        by[c].push_back(p[1]);
        bz[c].push_back(p[2]);
      }
    }
    fwgrid.start.assign(ncell + 1, 0);
    for (int c = 0; c < ncell; ++c) {
      fwgrid.start[c + 1] = fwgrid.start[c] + (int)bx[c].size();
      fwgrid.x.insert(fwgrid.x.end(), bx[c].begin(), bx[c].end());
      fwgrid.y.insert(fwgrid.y.end(), by[c].begin(), by[c].end());
      fwgrid.z.insert(fwgrid.z.end(), bz[c].begin(), bz[c].end());
    }
  }
  const double lim = overlap * (1.0 - 1.0e-9);
  for (int i = 1; i <= natms; ++i) {
    const double p[3] = {newx[i], newy[i], newz[i]};
    int c3[3];
    for (int d = 0; d < 3; ++d) {
      const double w = p[d] - L[d] * std::floor(p[d] / L[d]);
      c3[d] = std::min(fwgrid.nc[d] - 1, std::max(0, (int)(w / fwgrid.csz[d])));
    }
    for (int ox = -1; ox <= 1; ++ox)
      for (int oy = -1; oy <= 1; ++oy)
        for (int oz = -1; oz <= 1; ++oz) {
          const int cx = (c3[0] + ox + fwgrid.nc[0]) % fwgrid.nc[0];
          const int cy = (c3[1] + oy + fwgrid.nc[1]) % fwgrid.nc[1];
          const int cz = (c3[2] + oz + fwgrid.nc[2]) % fwgrid.nc[2];
          const int c = (cx * fwgrid.nc[1] + cy) * fwgrid.nc[2] + cz;
          for (int a = fwgrid.start[c]; a < fwgrid.start[c + 1]; ++a) {
            double dx = p[0] - fwgrid.x[a], dy = p[1] - fwgrid.y[a], dz = p[2] - fwgrid.z[a];
            images(imcon, 1, cell, &dx, &dy, &dz);
            const double rsq = dx * dx + dy * dy + dz * dz;
            if (rsq < lim) return true;
          }
        }
  }
  return false;
}

// insert_guests (mc_moves.f:84-149)
int Sim::insert_guests(int iguest, int nguests) {
  int m0 = locguest[iguest];
  long long maxiter = 1000LL * nguests;
  int iter = 0;
  if (mol[m0].nummols >= nguests) return 0;
  while (mol[m0].nummols < nguests) {
    if (iter >= maxiter) fail("oracle: insert_guests iteration cap (error 2320)");
    random_ins(iguest);
    if (prefilter_inserts && fw_overlap_certain(mol[m0].natoms)) {
      ++iter;  // insertion() would exit on this overlap; nothing to undo
      continue;
    }
    double estep = 0.0, delrc = 0.0, chgtmp = 0.0, engsictmp = 0.0;
    bool loverlap = false, lnewsurf = false;
    engsicorig = engsic;
    insertion(iguest, delrc, estep, chgtmp, engsictmp, loverlap, lnewsurf, nullptr);
    if (!loverlap) {
      int idum = 0;
      accept_move(iguest, true, false, false, lnewsurf, delrc, idum, engsictmp, chgtmp);
    } else {
      engsic = engsicorig;
    }
    std::fill(delE.begin(), delE.end(), 0.0);
    ++iter;
  }
  return iter;
}

}  // namespace

struct orc_sim {
  Sim s;
  std::unique_ptr<Sim> saved;  // orc_save_state
};

namespace {
template <class F>
int guarded(F &&f) {
  try {
    g_err.clear();
    return f();
  } catch (const std::exception &e) {
    g_err = e.what();
    return -1;
  }
}
}  // namespace

extern "C" {

const char *orc_last_error(void) { return g_err.c_str(); }

orc_sim *orc_create(const char *dir) {
  orc_sim *h = new orc_sim();
  int rc = guarded([&] {
    h->s.read_all(dir ? dir : ".");
    return 0;
  });
  if (rc != 0) {
    delete h;
    return nullptr;
  }
  return h;
}

void orc_destroy(orc_sim *h) { delete h; }

void orc_setup_energies(const orc_sim *h, double *out) {
  const Sim &s = h->s;
  out[0] = s.spe_vdw;
  out[1] = s.spe_ecoul / s.engunit;
  out[2] = s.spe_dlpeng / s.engunit;
  out[3] = s.ewald1sum;
  out[4] = s.alpha;
  out[5] = s.kmax1;
  out[6] = s.kmax2;
  out[7] = s.kmax3;
  out[8] = s.newld;
  out[9] = s.volm;
  out[10] = s.engunit;
  out[11] = s.sumchg;
  out[12] = std::sqrt(s.overlap);
}

void orc_seed(orc_sim *h, long long seed) {
  int ms, sec;
  seed_to_clock(seed, ms, sec);
  h->s.rng.init_from_clock(ms, sec);
}

int orc_ntpguest(const orc_sim *h) { return h->s.ntpguest; }
int orc_maxmls(const orc_sim *h) { return h->s.maxmls; }
int orc_nummols(const orc_sim *h, int m) { return h->s.mol[m].nummols; }
int orc_numatoms(const orc_sim *h, int m) { return h->s.mol[m].natoms; }
int orc_locguest(const orc_sim *h, int ig) { return h->s.locguest[ig]; }
int orc_newld(const orc_sim *h) { return h->s.newld; }
double orc_energy(const orc_sim *h, int m) { return h->s.energy[m]; }

int orc_get_coords(const orc_sim *h, int m, double *out, int cap) {
  const MolType &mt = h->s.mol[m];
  int n = mt.nummols * mt.natoms;
  for (int i = 1; i <= n && i <= cap; ++i) {
    out[3 * (i - 1) + 0] = mt.mx[i];
    out[3 * (i - 1) + 1] = mt.my[i];
    out[3 * (i - 1) + 2] = mt.mz[i];
  }
  return n;
}

int orc_get_sk(const orc_sim *h, double *out, int cap) {
  const Sim &s = h->s;
  int nm = s.maxmls + 1;
  int need = 2 * nm * s.newld;
  if (cap < need) return -need;
  for (int k = 1; k <= s.newld; ++k)
    for (int i = 1; i <= nm; ++i) {
      size_t idx = (size_t)(i - 1) + (size_t)(k - 1) * nm;
      out[2 * ((size_t)(k - 1) * nm + (i - 1)) + 0] = s.ckcsum[idx];
      out[2 * ((size_t)(k - 1) * nm + (i - 1)) + 1] = s.ckssum[idx];
    }
  return s.newld;
}

int orc_run(orc_sim *h, int nsteps, orc_move_log *log, int cap) {
  return guarded([&] {
    for (int i = 0; i < nsteps; ++i) h->s.step(log && i < cap ? &log[i] : nullptr);
    return nsteps;
  });
}

int orc_create_molecules(orc_sim *h, int iguest, int nguests) {
  return guarded([&] { return h->s.insert_guests(iguest, nguests); });
}

void orc_set_prefilter(orc_sim *h, int on) { h->s.prefilter_inserts = on != 0; }

// The set-up arrays the library's fmc_upload_system takes, by the name of
// its descriptor field, as doubles (0-based copies of the 1-based arrays,
// 2-D arrays column-major): the oracle stands in for a host that has done
// the reference's start-up.  Returns the element count (out == NULL: the
// count only), -count when cap is too small, -1 for an unknown name.
int orc_get_array(const orc_sim *h, const char *name, double *out, int cap) {
  const Sim &s = h->s;
  std::vector<double> v;
  const std::string n = name ? name : "";
  const int G = s.ntpguest;
  auto per_site = [&](auto get) {
    for (int m = 1; m <= s.maxmls; ++m)
      for (int a = 1; a <= s.mol[m].natoms; ++a) v.push_back(get(s.mol[m], a));
  };
  if (n == "imcon") v = {double(s.imcon)};
  else if (n == "cell") v.assign(s.cell, s.cell + 9);
  else if (n == "engunit") v = {s.engunit};
  else if (n == "temp") v = {s.temp};
  else if (n == "rcut") v = {s.rcut};
  else if (n == "alpha") v = {s.alpha};
  else if (n == "kmax") v = {double(s.kmax1), double(s.kmax2), double(s.kmax3)};
  else if (n == "newld") v = {double(s.newld)};
  else if (n == "epsq") v = {s.epsq};
  else if (n == "overlap") v = {std::sqrt(s.overlap)};
  else if (n == "surftol") v = {s.surftol};
  else if (n == "eqsteps") v = {double(s.eqsteps)};
  else if (n == "nwindsteps") v = {double(s.nwindsteps)};
  else if (n == "minchk") v = {double(s.minchk)};
  else if (n == "laccsample") v = {s.laccsample ? 1.0 : 0.0};
  else if (n == "ntpatm") v = {double(s.ntpatm)};
  else if (n == "mxegrd") v = {double(s.mxegrd)};
  else if (n == "drewd") v = {s.drewd};
  else if (n == "dlrpot") v = {s.dlrpot};
  else if (n == "erc") v.assign(s.erc.begin() + 1, s.erc.begin() + 1 + s.mxegrd);
  else if (n == "ntpvdw") v = {double(s.ntpvdw)};
  else if (n == "vvv") {
    for (int k = 1; k <= s.ntpvdw; ++k)
      for (int i = 1; i <= s.mxegrd; ++i) v.push_back(s.vvv[k][i]);
  } else if (n == "ltpvdw") {
    for (int k = 1; k <= s.ntpvdw; ++k) v.push_back(s.ltpvdw[k]);
  } else if (n == "prmvdw") {
    for (int c = 1; c <= 2; ++c)
      for (int k = 1; k <= s.ntpvdw; ++k) v.push_back(s.prmvdw[k][c]);
  } else if (n == "lstvdw" || n == "steadd") {
    const int np = s.ntpatm * (s.ntpatm + 1) / 2;
    for (int p = 1; p <= np; ++p) v.push_back(n == "lstvdw" ? double(s.lstvdw[p]) : s.steadd[p]);
  } else if (n == "maxmls") v = {double(s.maxmls)};
  else if (n == "numatoms" || n == "nummols" || n == "is_guest") {
    for (int m = 1; m <= s.maxmls; ++m)
      v.push_back(n == "numatoms" ? s.mol[m].natoms
                  : n == "nummols" ? s.mol[m].nummols : (s.mol[m].guest ? 1 : 0));
  } else if (n == "ltype") per_site([](const MolType &m, int a) { return double(m.ltp[a]); });
  else if (n == "charge") per_site([](const MolType &m, int a) { return m.chg[a]; });
  else if (n == "mass") per_site([](const MolType &m, int a) { return m.wght[a]; });
  else if (n == "frozen") per_site([](const MolType &m, int a) { return double(m.frz[a]); });
  else if (n == "fw_xyz") {
    for (int m = 1; m <= s.maxmls; ++m)
      if (!s.mol[m].guest)
        for (int i = 1; i <= s.mol[m].nummols * s.mol[m].natoms; ++i) {
          v.push_back(s.mol[m].mx[i]);
          v.push_back(s.mol[m].my[i]);
          v.push_back(s.mol[m].mz[i]);
        }
  } else if (n == "ntpguest") v = {double(G)};
  else if (n == "guest_tmpl") {
    for (int g = 1; g <= G; ++g)
      for (int i = 1; i <= s.mol[s.locguest[g]].natoms; ++i) {
        v.push_back(s.guestx[g][i]);
        v.push_back(s.guesty[g][i]);
        v.push_back(s.guestz[g][i]);
      }
  } else if (n == "fugacity" || n == "delr" || n == "disp_ratio" || n == "tran_ratio" ||
             n == "rota_ratio") {
    const std::vector<double> &a = n == "fugacity" ? s.gstfuga : n == "delr" ? s.delr
                                   : n == "disp_ratio" ? s.disp_ratio
                                   : n == "tran_ratio" ? s.tran_ratio : s.rota_ratio;
    for (int g = 1; g <= G; ++g) v.push_back(a[g]);
  } else if (n == "move_freq") {
    for (int g = 1; g <= G; ++g)
      for (const auto *a : {&s.mcinsf, &s.mcdelf, &s.mcdisf, &s.mcjmpf, &s.mcswpf, &s.mctraf,
                            &s.mcrotf, &s.mcswif})
        v.push_back((*a)[g]);
  } else if (n == "create") {
    for (int g = 1; g <= G; ++g) v.push_back(s.guest_insert[g]);
  } else {
    return -1;
  }
  const int cnt = (int)v.size();
  if (!out) return cnt;  // size query
  if (cap < cnt) return -cnt;
  for (int i = 0; i < cnt; ++i) out[i] = v[i];
  return cnt;
}

int orc_save_state(orc_sim *h) {
  return guarded([&] {
    h->saved = std::make_unique<Sim>(h->s);
    return 0;
  });
}

int orc_restore_state(orc_sim *h) {
  return guarded([&] {
    if (!h->saved) fail("oracle: no saved state");
    h->s = *h->saved;
    return 0;
  });
}

static void pack_out(Sim &s, int m0, double estep, double *parts, double delrc,
                     bool ov, bool sf, double *out) {
  out[0] = estep;
  out[1] = parts[0];
  out[2] = parts[1];
  out[3] = parts[2];
  out[4] = delrc;
  out[5] = ov;
  out[6] = sf;
  for (int i = 1; i <= s.maxmls; ++i) out[6 + i] = s.delE[i];
  (void)m0;
}

int orc_insertion_energy(orc_sim *h, int iguest, const double *xyz, double *out) {
  return guarded([&] {
    Sim &s = h->s;
    int m0 = s.locguest[iguest];
    int natms = s.mol[m0].natoms;
    for (int i = 1; i <= natms; ++i) {
      s.newx[i] = xyz[3 * (i - 1)];
      s.newy[i] = xyz[3 * (i - 1) + 1];
      s.newz[i] = xyz[3 * (i - 1) + 2];
    }
    double estep = 0, delrc = 0, chgtmp = 0, engsictmp = 0, parts[3] = {0, 0, 0};
    bool ov = false, sf = false;
    std::vector<double> esave = s.engsic;
    s.insertion(iguest, delrc, estep, chgtmp, engsictmp, ov, sf, parts);
    s.engsic = esave;
    pack_out(s, m0, estep, parts, delrc, ov, sf, out);
    return 0;
  });
}

int orc_deletion_energy(orc_sim *h, int iguest, int choice, double *out) {
  return guarded([&] {
    Sim &s = h->s;
    int m0 = s.locguest[iguest];
    if (choice < 1 || choice > s.mol[m0].nummols) fail("oracle: bad choice");
    double estep = 0, delrc = 0, chgtmp = 0, engsictmp = 0, parts[3] = {0, 0, 0};
    bool sf = false;
    s.deletion(iguest, choice, delrc, estep, sf, engsictmp, chgtmp, parts);
    pack_out(s, m0, estep, parts, delrc, false, sf, out);
    return 0;
  });
}

int orc_displace_energy(orc_sim *h, int iguest, int choice, const double *p,
                        double *out) {
  return guarded([&] {
    Sim &s = h->s;
    int m0 = s.locguest[iguest];
    if (choice < 1 || choice > s.mol[m0].nummols) fail("oracle: bad choice");
    std::vector<double> c0 = s.ckcsum, s0 = s.ckssum;
    bool li = false, ln = false, ov = false;
    double estep = 0.0;
    s.displace_guest(iguest, choice, p[0], p[1], p[2], p[3], p[4], p[5], p[6],
                     li, ln, ov, estep);
    s.ckcsum = c0;
    s.ckssum = s0;
    double parts[3] = {0, 0, 0};
    pack_out(s, m0, estep, parts, 0.0, ov, ln, out);
    return 0;
  });
}

int orc_apply_move(orc_sim *h, int kind, int iguest, int choice, const double *p,
                   int accepted) {
  return guarded([&] {
    Sim &s = h->s;
    int m0 = s.locguest[iguest];
    int natms = s.mol[m0].natoms;
    if (kind == 1) {
      for (int i = 1; i <= natms; ++i) {
        s.newx[i] = p[3 * (i - 1)];
        s.newy[i] = p[3 * (i - 1) + 1];
        s.newz[i] = p[3 * (i - 1) + 2];
      }
      s.engsicorig = s.engsic;
      double estep = 0, delrc = 0, chgtmp = 0, engsictmp = 0;
      bool ov = false, sf = false;
      s.insertion(iguest, delrc, estep, chgtmp, engsictmp, ov, sf, nullptr);
      if (accepted && !ov) {
        int rc = 0;
        s.accept_move(iguest, true, false, false, sf, delrc, rc, engsictmp, chgtmp);
      } else {
        s.reject_move(iguest, true, false, false);
      }
    } else if (kind == 2) {
      s.engsicorig = s.engsic;
      double estep = 0, delrc = 0, chgtmp = 0, engsictmp = 0;
      bool sf = false;
      s.deletion(iguest, choice, delrc, estep, sf, engsictmp, chgtmp, nullptr);
      if (accepted) {
        int rc = choice;
        s.accept_move(iguest, false, true, false, sf, delrc, rc, engsictmp, chgtmp);
      } else {
        s.reject_move(iguest, false, true, false);
      }
    } else if (kind == 3) {
      std::vector<double> c0 = s.ckcsum, s0 = s.ckssum;
      bool li = false, ln = false, ov = false;
      double estep = 0.0;
      s.displace_guest(iguest, choice, p[0], p[1], p[2], p[3], p[4], p[5], p[6],
                       li, ln, ov, estep);
      if (accepted && !ov) {
        int rc = choice;
        s.accept_move(iguest, false, false, true, ln, 0.0, rc, 0.0, 0.0);
      } else {
        s.ckcsum = c0;
        s.ckssum = s0;
        s.reject_move(iguest, false, false, true);
      }
    } else {
      fail("oracle: bad move kind");
    }
    return 0;
  });
}

int orc_prob_info(const orc_sim *h, int *out4) {
  const Sim &s = h->s;
  out4[0] = s.ngrida;
  out4[1] = s.ngridb;
  out4[2] = s.ngridc;
  out4[3] = s.lprob ? s.ntprob : 0;
  return 0;
}

int orc_prob_grid(const orc_sim *h, int sub, double *out, int n) {
  return guarded([&] {
    const Sim &s = h->s;
    if (!s.lprob || sub < 1 || sub > s.ntprob || n < s.gridsize) fail("oracle: bad probability grid request");
    std::copy(s.grid.begin() + (size_t)(sub - 1) * s.gridsize,
              s.grid.begin() + (size_t)sub * s.gridsize, out);
    return 0;
  });
}

// storeenprob (utility_pack.f:550-618) of given site coordinates and
// energy, as widom_grid calls it for a test insertion (gcmc.f:2529-2532).
int orc_store_energy(orc_sim *h, int iguest, const double *xyz, double energy) {
  return guarded([&] {
    Sim &s = h->s;
    if (!s.lprob || iguest < 1 || iguest > s.ntpguest || !s.lprobeng[iguest])
      fail("oracle: no energy probability grid for this guest type");
    const int n = s.mol[s.locguest[iguest]].natoms;
    for (int a = 1; a <= n; ++a) {
      s.newx[a] = xyz[3 * (a - 1)];
      s.newy[a] = xyz[3 * (a - 1) + 1];
      s.newz[a] = xyz[3 * (a - 1) + 2];
    }
    s.storeenprob(iguest, energy);
    return 0;
  });
}

long long orc_prodcount(const orc_sim *h) { return h->s.prodcount; }

double orc_fugacity(const orc_sim *h, int iguest) {
  const Sim &s = h->s;
  return iguest >= 1 && iguest <= s.ntpguest ? s.gstfuga[iguest] : -1.0;
}

int orc_swap(orc_sim *h, int iguest, int choice, int jguest, const double *q,
             const double *rande, double *out) {
  return guarded([&] {
    Sim &s = h->s;
    if (iguest < 1 || iguest > s.ntpguest || jguest < 1 || jguest > s.ntpguest ||
        jguest == iguest)
      fail("orc_swap: bad guest types");
    if (choice < 1 || choice > s.mol[s.locguest[iguest]].nummols)
      fail("orc_swap: bad molecule");
    const bool prod = s.production;
    s.production = false;  // a stand-alone swap adds no production sample
    s.swap_move(iguest, choice, jguest, q, rande, out, nullptr);
    s.production = prod;
    return 0;
  });
}

void orc_stats(const orc_sim *h, int ig, double *out) {
  const Sim &s = h->s;
  int vs = 1 + (ig - 1) * 9;
  double sw = 0, acc[9] = {0};
  for (const auto &w : s.avgwindow) {
    sw += w[1];
    for (int q = 1; q <= 8; ++q) acc[q] += w[1] * w[vs + q];
  }
  for (int q = 1; q <= 8; ++q) out[q - 1] = sw > 0 ? acc[q] / sw : 0.0;
  out[8] = double(s.prodcount);
  out[9] = double(s.avgwindow.size());
  out[10] = (double)s.ins_count[ig];
  out[11] = (double)s.accept_ins[ig];
  out[12] = (double)s.del_count[ig];
  out[13] = (double)s.accept_del[ig];
  out[14] = (double)s.disp_count[ig];
  out[15] = (double)s.accept_disp[ig];
  out[16] = (double)s.rota_count[ig];
  out[17] = (double)s.accept_rota[ig];
  out[18] = (double)s.tran_count[ig];
  out[19] = (double)s.accept_tran[ig];
  out[20] = s.delrdisp[ig];
  out[21] = s.rotangle;
  out[22] = s.rota_rotangle;
  out[23] = (double)s.jump_count[ig];
  out[24] = (double)s.accept_jump[ig];
  out[25] = (double)s.swap_count[ig];
  out[26] = (double)s.accept_swap[ig];
  out[27] = (double)s.switch_count[ig];
  out[28] = (double)s.accept_switch[ig];
  // "standard error" of <N> as the reference prints it (gcmc.f:1218-1241):
  // the weighted standard deviation of the window averages
  double sd = 0.0;
  for (const auto &w : s.avgwindow) {
    const double d = out[0] - w[vs + 1];
    sd += w[1] * d * d;
  }
  out[29] = sw > 0 ? std::sqrt(sd / sw) : 0.0;
}

void orc_duni_sequence(long long seed, int n, double *out) {
  Duni d;
  int ms, sec;
  seed_to_clock(seed, ms, sec);
  d.init_from_clock(ms, sec);
  for (int i = 0; i < n; ++i) out[i] = d.next();
}

int orc_get_erc(const orc_sim *h, double *out, int cap) {
  const Sim &s = h->s;
  for (int i = 1; i <= s.mxegrd && i <= cap; ++i) out[i - 1] = s.erc[i];
  return s.mxegrd;
}

int orc_get_vvv(const orc_sim *h, int k, double *out, int cap) {
  const Sim &s = h->s;
  if (k < 1 || k > s.maxvdw + 1) return -1;
  for (int i = 1; i <= s.mxegrd && i <= cap; ++i) out[i - 1] = s.vvv[k][i];
  return s.mxegrd;
}

}  // extern "C"

// host_setup.cpp -- start-up work the reference's Fortran host performs
// before the first trial move (gcmc.f:203-590), restated in C++ so the GPU
// path can be driven without a Fortran compiler.  The number parsing keeps
// the reference's rules (parse_module.f), so every constant matches what
// the Fortran host would hand to the ABI.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fmc_internal.h"

namespace fmc {
namespace {

constexpr int kLen = 150;  // lenrec (parse_module.f:9)

// A 150-column, blank-padded input record.
struct Record {
  char c[kLen];
  char &at(int i) { return c[i - 1]; }
  char at(int i) const { return c[i - 1]; }
};

class Reader {
 public:
  explicit Reader(const std::string &path) : path_(path) {
    f_ = std::fopen(path.c_str(), "r");
    if (!f_) raise(FMC_ERR_INPUT, "cannot open " + path);
  }
  ~Reader() {
    if (f_) std::fclose(f_);
  }
  // getrec (parse_module.f:15-79)
  bool get(Record &r) {
    char buf[4096];
    if (!std::fgets(buf, sizeof buf, f_)) return false;
    size_t n = std::strlen(buf);
    while (n && (buf[n - 1] == '\n' || buf[n - 1] == '\r')) --n;
    for (int i = 0; i < kLen; ++i) r.c[i] = size_t(i) < n ? buf[i] : ' ';
    return true;
  }
  void need(Record &r) {
    if (!get(r)) raise(FMC_ERR_INPUT, path_ + " ended early");
  }
  bool line(std::string &out) {
    char buf[4096];
    if (!std::fgets(buf, sizeof buf, f_)) return false;
    out = buf;
    while (!out.empty() && (out.back() == '\n' || out.back() == '\r')) out.pop_back();
    return true;
  }

 private:
  std::string path_;
  FILE *f_ = nullptr;
};

// lowcase / strip / findstring (parse_module.f:258-427)
void lower(Record &r, int n = kLen) {
  for (int i = 1; i <= std::min(n, kLen); ++i)
    if (r.at(i) >= 'A' && r.at(i) <= 'Z') r.at(i) = char(r.at(i) + 32);
}
void strip_lead(Record &r, int n = kLen) {
  int k = 0;
  while (k < n && r.c[k] == ' ') ++k;
  if (k == 0) return;
  for (int i = 0; i < n; ++i) r.c[i] = (i + k < n) ? r.c[i + k] : ' ';
}
bool has(const Record &r, const char *s) {
  int n = (int)std::strlen(s);
  for (int h = 0; h + n <= kLen; ++h)
    if (std::memcmp(r.c + h, s, n) == 0) return true;
  return false;
}
void consume(char *w, int len, int lst) {
  for (int j = lst; j <= len; ++j) w[j - lst] = w[j - 1];
  for (int j = len - lst + 2; j <= len; ++j) w[j - 1] = ' ';
}
// intstr (parse_module.f:81-146)
int int_of(char *w, int len, int *used = nullptr) {
  int sign = 1, v = 0, lst = 0;
  bool seen = false, done = false;
  char prev = '+';
  while (lst < len && !done) {
    char ch = w[lst++];
    bool dig = ch >= '0' && ch <= '9';
    if (dig) {
      v = 10 * v + (ch - '0');
      seen = true;
    }
    if (seen && !dig) done = true;
    if (dig && prev == '-') sign = -1;
    prev = ch;
  }
  consume(w, len, lst);
  if (used) *used = lst;
  return sign * v;
}
int int_of(Record &r) { return int_of(r.c, kLen); }
// dblstr (parse_module.f:148-256): digits accumulate as ten*v + one*d.
double dbl_of(char *w, int len) {
  int lst = 0, iexp = 0, used = 0;
  double sign = 1.0, ten = 10.0, one = 1.0, v = 0.0;
  bool started = false, dot = false, done = false;
  char prev = '+';
  while (lst < len && !done) {
    ++lst;
    char ch = w[lst - 1];
    bool flag = false;
    if (ch >= '0' && ch <= '9') {
      double a = ten * v;
      double b = one * double(ch - '0');
      v = a + b;
      flag = started = true;
    }
    if (ch == '.') {
      flag = started = dot = true;
      ten = 1.0;
    }
    if (flag && prev == '-') sign = -1.0;
    if (dot) one = one / 10.0;
    prev = ch;
    if (prev == 'D') prev = 'd';
    if (prev == 'E') prev = 'e';
    if (started) {
      if (prev == 'd' || prev == 'e') {
        std::vector<char> tail(std::max(1, len - lst), ' ');
        for (int i = 0; i < len - lst; ++i) tail[i] = w[lst + i];
        iexp = int_of(tail.data(), len - lst, &used);
        done = true;
      }
      if (!flag) done = true;
    }
  }
  double p = 1.0;
  for (int i = 0; i < std::abs(iexp); ++i) p *= 10.0;
  if (iexp < 0) p = 1.0 / p;
  v = sign * v * p;
  consume(w, len, lst + used);
  return v;
}
double dbl_of(Record &r) { return dbl_of(r.c, kLen); }
// getword (parse_module.f:547-602)
std::string word_of(Record &r, int maxlen) {
  std::string w;
  int i = 0;
  bool done = false;
  while (!done && i < kLen) {
    ++i;
    char ch = r.c[0];
    if (ch == ' ') {
      if (!w.empty()) done = true;
    } else {
      w.push_back(ch);
      if ((int)w.size() == maxlen) done = true;
    }
    std::memmove(r.c, r.c + 1, kLen - 1);
    r.c[kLen - 1] = ' ';
  }
  w.resize(8, ' ');
  return w;
}

std::string join(const std::string &d, const char *f) { return d.empty() ? f : d + "/" + f; }

void invert3(const double *a, double *b) {
  b[0] = a[4] * a[8] - a[5] * a[7];
  b[1] = a[2] * a[7] - a[1] * a[8];
  b[2] = a[1] * a[5] - a[2] * a[4];
  b[3] = a[5] * a[6] - a[3] * a[8];
  b[4] = a[0] * a[8] - a[2] * a[6];
  b[5] = a[2] * a[3] - a[0] * a[5];
  b[6] = a[3] * a[7] - a[4] * a[6];
  b[7] = a[1] * a[6] - a[0] * a[7];
  b[8] = a[0] * a[4] - a[1] * a[3];
  double d = a[0] * b[0] + a[3] * b[1] + a[6] * b[2];
  double r = std::fabs(d) > 0.0 ? 1.0 / d : 0.0;
  for (int i = 0; i < 9; ++i) b[i] *= r;
}

// dcell (utility_pack.f:1904-1960)
void cell_props(const double *a, double *b) {
  b[0] = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  b[1] = std::sqrt(a[3] * a[3] + a[4] * a[4] + a[5] * a[5]);
  b[2] = std::sqrt(a[6] * a[6] + a[7] * a[7] + a[8] * a[8]);
  b[3] = (a[0] * a[3] + a[1] * a[4] + a[2] * a[5]) / (b[0] * b[1]);
  b[4] = (a[0] * a[6] + a[1] * a[7] + a[2] * a[8]) / (b[0] * b[2]);
  b[5] = (a[3] * a[6] + a[4] * a[7] + a[5] * a[8]) / (b[1] * b[2]);
  double axb[3] = {a[1] * a[5] - a[2] * a[4], a[2] * a[3] - a[0] * a[5],
                   a[0] * a[4] - a[1] * a[3]};
  double bxc[3] = {a[4] * a[8] - a[5] * a[7], a[5] * a[6] - a[3] * a[8],
                   a[3] * a[7] - a[4] * a[6]};
  double cxa[3] = {a[7] * a[2] - a[1] * a[8], a[0] * a[8] - a[2] * a[6],
                   a[1] * a[6] - a[0] * a[7]};
  b[9] = std::fabs(a[0] * bxc[0] + a[1] * bxc[1] + a[2] * bxc[2]);
  b[6] = b[9] / std::sqrt(bxc[0] * bxc[0] + bxc[1] * bxc[1] + bxc[2] * bxc[2]);
  b[7] = b[9] / std::sqrt(cxa[0] * cxa[0] + cxa[1] * cxa[1] + cxa[2] * cxa[2]);
  b[8] = b[9] / std::sqrt(axb[0] * axb[0] + axb[1] * axb[1] + axb[2] * axb[2]);
}

// Minimum image of one vector (utility_pack.f:1697-1791, imcon 1-3).
void min_image(const System &s, double &x, double &y, double &z) {
  if (s.imcon == 1) {
    double a = 1.0 / s.cell[0];
    x -= s.cell[0] * std::round(a * x);
    y -= s.cell[0] * std::round(a * y);
    z -= s.cell[0] * std::round(a * z);
  } else if (s.imcon == 2) {
    x -= s.cell[0] * std::round((1.0 / s.cell[0]) * x);
    y -= s.cell[4] * std::round((1.0 / s.cell[4]) * y);
    z -= s.cell[8] * std::round((1.0 / s.cell[8]) * z);
  } else if (s.imcon == 3) {
    const double *r = s.rcell, *c = s.cell;
    double sx = r[0] * x + r[3] * y + r[6] * z;
    double sy = r[1] * x + r[4] * y + r[7] * z;
    double sz = r[2] * x + r[5] * y + r[8] * z;
    sx -= std::round(sx);
    sy -= std::round(sy);
    sz -= std::round(sz);
    x = c[0] * sx + c[3] * sy + c[6] * sz;
    y = c[1] * sx + c[4] * sy + c[7] * sz;
    z = c[2] * sx + c[5] * sy + c[8] * sz;
  }
}

// --- initscan (utility_pack.f:207-508): sizes, cell, cutoff, Ewald ----------
void scan_inputs(const std::string &dir, System &s) {
  Record r;
  std::vector<std::string> names;
  {
    Reader f(join(dir, "FIELD"));
    f.need(r);
    for (;;) {
      f.need(r);
      lower(r);
      strip_lead(r);
      if (r.c[0] == '#' || r.c[0] == ' ') continue;
      if (has(r, "molecu")) {
        s.maxmls = int_of(r);
        for (int n = 0; n < s.maxmls; ++n) {
          for (;;) {
            f.need(r);
            lower(r);
            strip_lead(r);
            if (r.c[0] == '#' || r.c[0] == ' ') continue;
            if (has(r, "nummol")) continue;
            if (has(r, "atoms")) {
              int nsit = int_of(r), k = 0;
              for (int i = 0; i < nsit; ++i) {
                if (k >= nsit) continue;
                f.need(r);
                std::string nm = word_of(r, 8);
                dbl_of(r);
                dbl_of(r);
                int nrept = int_of(r);
                if (nrept == 0) nrept = 1;
                k += nrept;
                if (std::find(names.begin(), names.end(), nm) == names.end())
                  names.push_back(nm);
              }
            } else if (has(r, "finish")) {
              break;
            }
          }
        }
      } else if (has(r, "vdw")) {
        s.ntpvdw = int_of(r);
      } else if (has(r, "close")) {
        break;
      }
    }
  }
  s.mxatyp = (int)names.size();
  {
    Reader f(join(dir, "CONFIG"));
    f.need(r);
    f.need(r);
    s.imcon = int_of(r);
    s.imcon = int_of(r);
    for (int row = 0; row < 3; ++row) {
      f.need(r);
      for (int j = 0; j < 3; ++j) s.cell[3 * row + j] = dbl_of(r);
    }
  }
  cell_props(s.cell, s.celprp);
  bool lcut = false, ldelr = false, lwind = false, lrvdw = false, lewald = false;
  {
    Reader f(join(dir, "CONTROL"));
    for (;;) {
      f.need(r);
      lower(r);
      strip_lead(r);
      if (r.c[0] == '#' || r.c[0] == ' ') continue;
      if (has(r, "cut")) {
        s.rcut = dbl_of(r);
        lcut = true;
      } else if (has(r, "&guest")) {
        for (;;) {
          f.need(r);
          lower(r);
          strip_lead(r);
          if (r.c[0] == '#' || r.c[0] == ' ') continue;
          if (has(r, "probability")) {  // utility_pack.f:360-380
            int q = int_of(r), got = 0;
            s.lprob = true;
            s.ntprob += q;
            while (got < q) {
              f.need(r);
              strip_lead(r);
              if (r.c[0] == '#' || r.c[0] == ' ') continue;
              if (r.c[0] == 'e') ++s.ntprob;  // energy grid: one more
              ++got;
            }
          } else if (has(r, "&end")) {
            break;
          }
        }
      } else if (has(r, "henry")) {
      } else if (has(r, "grid")) {  // utility_pack.f:436-443
        if (has(r, "spa")) {
          s.griddim = dbl_of(r);
        } else if (has(r, "fac")) {
          for (int d = 0; d < 3; ++d) s.gridfactor[d] = int_of(r);
        }
      } else if (has(r, "delr")) {
        s.initdelr = dbl_of(r);
        ldelr = true;
      } else if (has(r, "averaging window")) {
        s.nwind = int_of(r);
        lwind = true;
      } else if (has(r, "steps")) {
        s.mcsteps = int_of(r);
      } else if (has(r, "finish")) {
        break;
      } else if (has(r, "ewald")) {
        lewald = true;
        if (has(r, "precision")) {
          if (!lcut) raise(FMC_ERR_INPUT, "ewald precision before cutoff (error 433)");
          double eps = std::min(std::fabs(dbl_of(r)), 0.5);
          double tol = std::sqrt(std::fabs(std::log(eps * s.rcut)));
          s.alpha = std::sqrt(std::fabs(std::log(eps * s.rcut * tol))) / s.rcut;
          double t = 2.0 * tol * s.alpha;
          double tol1 = std::sqrt(-std::log(eps * s.rcut * (t * t)));
          for (int d = 0; d < 3; ++d)
            s.kmax[d] = (int)std::round(0.25 + s.celprp[d] * s.alpha * tol1 / kPi);
        } else {
          s.alpha = dbl_of(r);
          for (int d = 0; d < 3; ++d) s.kmax[d] = int_of(r);
        }
      } else if (has(r, "rvdw")) {
        s.rvdw = dbl_of(r);
        lrvdw = true;
      }
    }
  }
  if (!ldelr) raise(FMC_ERR_INPUT, "CONTROL has no delr (error 433)");
  if (!lewald) raise(FMC_ERR_INPUT, "CONTROL has no ewald directive (error 2311)");
  if (s.imcon < 1 || s.imcon > 3)
    raise(FMC_ERR_INPUT, "only imcon 1, 2 and 3 are supported");
  int cf = std::abs(s.mcsteps);
  if (!lwind) s.nwind = cf > 1000 ? 5 : 1;
  s.nwindsteps = std::max(1, (int)std::ceil(double(cf) / double(s.nwind)));
  double width = std::min(s.celprp[6], std::min(s.celprp[7], s.celprp[8])) / 2.0;
  if (s.rcut > width) raise(FMC_ERR_INPUT, "cutoff exceeds half the cell width (error 95)");
  s.volm = s.celprp[9];
  if (!lrvdw && s.rcut > 0.0) s.rvdw = s.rcut;
  s.maxvdw = std::max(s.ntpvdw, (s.mxatyp * (s.mxatyp + 1)) / 2);
  s.mxegrd = std::max(1000, int(s.rvdw / 0.01 + 0.5) + 4);
}

// --- readfield (readinputs.f:11-307) + define_van_der_waals --------------
void read_field(const std::string &dir, System &s) {
  Record r;
  Reader f(join(dir, "FIELD"));
  s.mol.assign(s.maxmls + 1, MolType());
  s.locguest.assign(1, 0);
  s.locfram.assign(1, 0);
  s.unqatm.assign(1, "");
  s.guest_tmpl.assign(1, {});
  s.ltpvdw.assign(s.maxvdw + 2, -1);
  s.lstvdw.assign(s.maxvdw + 2, 0);
  s.prmvdw.assign(s.maxvdw + 2, std::array<double, 6>{0, 0, 0, 0, 0, 0});
  s.vvv.assign(s.maxvdw + 2, std::vector<double>(s.mxegrd + 3, 0.0));
  f.need(r);
  for (;;) {
    f.need(r);
    lower(r);
    strip_lead(r);
    if (has(r, "units")) {
      bool blank = true;
      for (int i = 6; i <= kLen; ++i)
        if (r.at(i) != ' ') blank = false;
      if (blank) {
      } else if (has(r, "ev")) s.engunit = 9648.530821;
      else if (has(r, "kcal")) s.engunit = 418.4;
      else if (has(r, "kj")) s.engunit = 1.0e2;
      else if (has(r, "k")) s.engunit = kBoltz;
    } else if (has(r, "vdw")) {
      for (int i = 1; i <= s.ntpvdw; ++i) {
        f.need(r);
        std::string a1 = word_of(r, 8), a2 = word_of(r, 8);
        lower(r, kLen - 16);
        std::string kw = word_of(r, 4).substr(0, 4);
        int key;
        if (kw == "12-6") key = 1;
        else if (kw == "lj  ") key = 2;
        else raise(FMC_ERR_INPUT, "only lj and 12-6 van der Waals forms are supported");
        std::array<double, 6> p{0, 0, 0, 0, 0, 0};
        for (int q = 1; q <= 5; ++q) p[q] = dbl_of(r);
        int k1 = 0, k2 = 0;
        for (int j = 1; j <= s.ntpatm; ++j) {
          if (a1 == s.unqatm[j]) k1 = j;
          if (a2 == s.unqatm[j]) k2 = j;
        }
        if (!k1 || !k2) raise(FMC_ERR_INPUT, "VDW line names an unknown atom");
        p[1] *= s.engunit;
        if (key == 1) p[2] *= s.engunit;
        s.lstvdw[loc2(k1, k2)] = i;
        s.ltpvdw[i] = key;
        s.prmvdw[i] = p;
      }
      // forgen (vdw_terms.f:181-234)
      s.dlrpot = s.rvdw / double(s.mxegrd - 4);
      for (int iv = 1; iv <= s.ntpvdw; ++iv)
        for (int i = 1; i <= s.mxegrd; ++i) {
          double rr = double(i) * s.dlrpot;
          if (s.ltpvdw[iv] == 1) {
            double r6 = std::pow(rr, 6);
            s.vvv[iv][i] = (s.prmvdw[iv][1] / r6 - s.prmvdw[iv][2]) / r6;
          } else {
            double sr6 = std::pow(s.prmvdw[iv][2] / rr, 6);
            s.vvv[iv][i] = 4.0 * s.prmvdw[iv][1] * sr6 * (sr6 - 1.0);
          }
        }
      int ntab = s.ntpatm * (s.ntpatm + 1) / 2;
      if (s.ntpvdw < ntab)
        for (int i = 1; i <= ntab; ++i)
          if (s.lstvdw[i] == 0) s.lstvdw[i] = s.ntpvdw + 1;
    } else if (has(r, "molecu")) {
      int ntpmls = int_of(r);
      if (ntpmls != s.maxmls) raise(FMC_ERR_INPUT, "molecule count mismatch");
      for (int n = 1; n <= ntpmls; ++n) {
        MolType &m = s.mol[n];
        f.need(r);
        lower(r);
        if (has(r, "&guest")) {
          m.guest = true;
          s.locguest.push_back(n);
          s.guest_tmpl.push_back({});
          ++s.ntpguest;
        } else {
          s.locfram.push_back(n);
          ++s.ntpfram;
        }
        m.name = std::string(r.c, 40);
        double mass = 0.0;
        for (;;) {
          f.need(r);
          lower(r);
          strip_lead(r);
          if (has(r, "nummol")) {
            m.nummols = int_of(r);
          } else if (has(r, "atoms")) {
            int ns = int_of(r);
            m.natoms = ns;
            m.site.assign(ns, "");
            m.wght.assign(ns, 0.0);
            m.chg.assign(ns, 0.0);
            m.frz.assign(ns, 0);
            m.ltp.assign(ns, 0);
            std::vector<double> tmpl(3 * ns, 0.0);
            int k = 0;
            while (k < ns) {
              f.need(r);
              std::string a = word_of(r, 8);
              double w = dbl_of(r), q = dbl_of(r);
              int nrept = 1, ifrz = 0;
              if (m.guest) {
                tmpl[3 * k] = dbl_of(r);
                tmpl[3 * k + 1] = dbl_of(r);
                tmpl[3 * k + 2] = dbl_of(r);
              } else {
                nrept = int_of(r);
                ifrz = int_of(r);
                if (nrept == 0) nrept = 1;
              }
              int type = 0;
              for (int j = 1; j <= s.ntpatm; ++j)
                if (s.unqatm[j] == a) type = j;
              if (!type) {
                s.unqatm.push_back(a);
                type = ++s.ntpatm;
              }
              for (int rp = 0; rp < nrept; ++rp) {
                if (k >= ns) raise(FMC_ERR_INPUT, "site repeat overflow");
                m.site[k] = a;
                m.wght[k] = w;
                m.chg[k] = q;
                m.frz[k] = ifrz;
                m.ltp[k] = type;
                mass += w;
                ++k;
              }
            }
            if (m.guest) s.guest_tmpl.back() = tmpl;
          } else if (has(r, "finish")) {
            if (m.guest) {
              // readinputs.f:221-243: the subtracted centre is
              // sum(m_i r_i) / (2 M) because the site masses are summed
              // twice.  Kept as the reference does it.
              auto &t = s.guest_tmpl.back();
              double c[3] = {0, 0, 0};
              for (int i = 0; i < m.natoms; ++i) {
                for (int d = 0; d < 3; ++d) c[d] += t[3 * i + d] * m.wght[i];
                mass += m.wght[i];
              }
              for (int d = 0; d < 3; ++d) c[d] /= mass;
              for (int i = 0; i < m.natoms; ++i)
                for (int d = 0; d < 3; ++d) t[3 * i + d] -= c[d];
            }
            break;
          }
        }
      }
    } else if (has(r, "close")) {
      break;
    } else {
      raise(FMC_ERR_INPUT, "unrecognised FIELD directive");
    }
  }
  s.sumchg = 0.0;
  for (int it = 1; it <= s.maxmls; ++it)
    for (int l = 0; l < s.mol[it].natoms; ++l)
      s.sumchg += double(s.mol[it].nummols) * s.mol[it].chg[l];
  if (s.ntpfram != 1) raise(FMC_ERR_INPUT, "exactly one framework molecule type is supported");
  if (s.ntpguest < 1 || s.ntpguest > FMC_MAX_GUEST_TYPES)
    raise(FMC_ERR_INPUT, "between 1 and 4 guest types are supported");
  if (s.maxmls > FMC_MAX_MOLTYPES) raise(FMC_ERR_INPUT, "too many molecule types");
  s.fw_mol = s.locfram[1];
  for (int g = 1; g <= s.ntpguest; ++g) {
    const MolType &m = s.mol[s.locguest[g]];
    if (m.natoms > FMC_MAX_SITES) raise(FMC_ERR_INPUT, "guest has too many sites");
    if (m.nummols != 0)
      raise(FMC_ERR_INPUT, "guests in CONFIG are not supported; use create molecules");
  }
  for (int k = 0; k < s.mol[s.fw_mol].natoms; ++k)
    if (s.mol[s.fw_mol].frz[k] == 0)
      raise(FMC_ERR_INPUT, "non-frozen framework atoms are not supported");
}

// --- readconfig (readinputs.f:309-513), levcfg 0-2, 3f20.0 fields -------
void read_config(const std::string &dir, System &s) {
  Record r;
  Reader f(join(dir, "CONFIG"));
  f.need(r);
  s.cfgname.assign(r.c, r.c + 80);  // cfgname, the title record's first 80 characters
  f.need(r);
  int levcfg = int_of(r);
  for (int row = 0; row < 3; ++row) {
    f.need(r);
    for (int j = 0; j < 3; ++j) s.cell[3 * row + j] = dbl_of(r);
  }
  auto fields3 = [&](double *v) {
    std::string ln;
    if (!f.line(ln)) raise(FMC_ERR_INPUT, "CONFIG truncated");
    ln.resize(60, ' ');
    for (int j = 0; j < 3; ++j) v[j] = std::strtod(ln.substr(20 * j, 20).c_str(), nullptr);
  };
  for (int k = 1; k <= s.maxmls; ++k) {
    MolType &m = s.mol[k];
    m.xyz.assign(3 * size_t(m.nummols) * m.natoms, 0.0);
    size_t idx = 0;
    for (int l = 0; l < m.nummols; ++l)
      for (int a = 0; a < m.natoms; ++a) {
        std::string nm;
        if (!f.line(nm)) raise(FMC_ERR_INPUT, "CONFIG truncated");
        nm.resize(8, ' ');
        size_t b = nm.find_first_not_of(' ');
        std::string name = b == std::string::npos ? std::string(8, ' ') : nm.substr(b);
        name.resize(8, ' ');
        double v[3], junk[3];
        fields3(v);
        if (levcfg >= 1) fields3(junk);
        if (levcfg >= 2) fields3(junk);
        if (name != m.site[a]) raise(FMC_ERR_INPUT, "unidentified atom label in CONFIG (error 25)");
        for (int d = 0; d < 3; ++d) m.xyz[idx++] = v[d];
      }
  }
  cell_props(s.cell, s.celprp);
  s.volm = s.celprp[9];
  invert3(s.cell, s.rcell);
  if (s.imcon == 2 || s.imcon == 1)
    for (int i : {1, 2, 3, 5, 6, 7})
      if (std::fabs(s.cell[i]) > 1e-10) raise(FMC_ERR_INPUT, "cell is not orthorhombic (error 410)");
}

// --- readcontrol (readinputs.f:515-944) ---------------------------------
void read_control(const std::string &dir, System &s) {
  Record r;
  Reader f(join(dir, "CONTROL"));
  int G = s.ntpguest;
  s.gstpress.assign(G + 1, -1.0);
  s.gstmolfract.assign(G + 1, -1.0);
  s.delr.assign(G + 1, s.initdelr);
  s.disp_ratio.assign(G + 1, 0.5);
  s.tran_ratio.assign(G + 1, 0.5);
  s.rota_ratio.assign(G + 1, 0.5);
  s.guest_insert.assign(G + 1, 0);
  std::vector<float> *mv[8] = {&s.mcinsf, &s.mcdelf, &s.mcdisf, &s.mcjmpf,
                               &s.mcswpf, &s.mcswif, &s.mctraf, &s.mcrotf};
  for (auto *v : mv) v->assign(G + 1, -1.0f);
  const char *keys[8] = {"ins", "del", "dis", "jum", "swa", "swi", "tra", "rot"};
  double glob[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
  bool ltemp = false, lsteps = false, leq = false, lnumg = false;
  int ngst = 0, piprob = 0;
  s.nprob.assign(G + 1, 0);
  s.lprobeng.assign(G + 1, 0);
  s.nprobsites.assign(s.ntprob + 1, 0);
  s.lprobsites.assign(s.ntprob + 1, std::vector<int>());
  f.need(r);
  for (;;) {
    f.need(r);
    lower(r);
    strip_lead(r);
    if (r.c[0] == '#' || r.c[0] == ' ') continue;
    if (has(r, "block")) raise(FMC_ERR_INPUT, "pore blocking is not supported");
    else if (has(r, "henry")) {
    } else if (has(r, "widom ins")) {
    } else if (has(r, "restart")) raise(FMC_ERR_INPUT, "restart is not supported");
    else if (has(r, "temp")) {
      s.temp = dbl_of(r);
      ltemp = true;
    } else if (has(r, "sampling")) {
      s.laccsample = true;
    } else if (has(r, "&guest")) {
      ++ngst;
      int g = int_of(r);
      if (g < 1 || g > G) raise(FMC_ERR_INPUT, "&guest index out of range");
      bool rprob = false;
      for (;;) {
        f.need(r);
        lower(r);
        strip_lead(r);
        if (r.c[0] == '#' || r.c[0] == ' ') continue;
        if (has(r, "fract")) s.gstmolfract[g] = dbl_of(r);
        else if (has(r, "create molecules")) s.guest_insert[g] = int_of(r);
        else if (has(r, "min molecules") || has(r, "max molecules")) int_of(r);
        else if (has(r, "press")) s.gstpress[g] = dbl_of(r) * 1.0e5;
        else if (has(r, "probability")) {  // readinputs.f:642-672
          rprob = true;
          bool leng = false;
          int q = int_of(r), got = 0;
          s.nprob[g] = q;
          while (got < q) {
            f.need(r);
            strip_lead(r);
            if (r.c[0] == '#' || r.c[0] == ' ') continue;
            ++got;
            if (r.c[0] == 'e') {
              leng = true;
              continue;
            }
            ++piprob;
            if (piprob > s.ntprob) raise(FMC_ERR_INPUT, "probability blocks inconsistent");
            const int nsite = int_of(r);
            s.nprobsites[piprob] = nsite;
            s.lprobsites[piprob].assign(nsite + 1, 0);
            for (int j = 1; j <= nsite; ++j) s.lprobsites[piprob][j] = int_of(r);
          }
          if (leng) {
            s.lprobeng[g] = 1;
            s.nprob[g] += 1;
          }
        } else if (has(r, "move")) {
          for (int q = 0; q < 8; ++q)
            if (has(r, keys[q])) {
              (*mv[q])[g] = (float)dbl_of(r);
              break;
            }
        } else if (has(r, "delr")) s.delr[g] = dbl_of(r);
        else if (has(r, "accep")) {
          if (has(r, "dis")) s.disp_ratio[g] = dbl_of(r);
          else if (has(r, "tra")) s.tran_ratio[g] = dbl_of(r);
        } else if (has(r, "&end")) break;
      }
      if (!rprob) s.nprob[ngst] = 0;  // readinputs.f:706 (indexed by the block count)
    } else if (has(r, "steps")) {
      s.mcsteps = int_of(r);
      lsteps = true;
    } else if (has(r, "pressure") || has(r, "total press")) {
      s.total_pressure = dbl_of(r) * 1.0e5;
    } else if (has(r, "numg")) {
      lnumg = true;
      s.nnumg = int_of(r);
      if (s.nnumg <= 0) s.nnumg = 1000;
    } else if (has(r, "fuga")) {
      s.lfuga = true;
    } else if (has(r, "hist")) {
    } else if (has(r, "equilibr")) {
      s.eqsteps = int_of(r);
      leq = s.eqsteps != 0;
    } else if (has(r, "wang-landau")) raise(FMC_ERR_INPUT, "Wang-Landau is not supported");
    else if (has(r, "uvt") || has(r, "single point")) {
    } else if (has(r, "jobcontrol")) raise(FMC_ERR_INPUT, "jobcontrol is not supported");
    else if (has(r, "cutoff")) s.rcut = dbl_of(r);
    else if (has(r, "overlap")) s.overlap_sq = dbl_of(r);
    else if (has(r, "surface")) s.surftol = dbl_of(r);
    else if (has(r, "delr")) dbl_of(r);
    else if (has(r, "averaging window") || has(r, "max")) {
    } else if (has(r, "move")) {
      for (int q = 0; q < 8; ++q)
        if (has(r, keys[q])) {
          glob[q] = dbl_of(r);
          break;
        }
    } else if (has(r, "accep") || has(r, "grid") || has(r, "ewald")) {
    } else if (has(r, "finish")) {
      break;
    } else {
      raise(FMC_ERR_INPUT, "unknown CONTROL directive (error 3)");
    }
  }
  if (ngst != G) raise(FMC_ERR_INPUT, "guest blocks do not match FIELD (error 2312)");
  if (!ltemp) raise(FMC_ERR_INPUT, "CONTROL has no temperature (error 380)");
  for (int g = 1; g <= G; ++g)
    for (int q = 0; q < 8; ++q)
      if ((*mv[q])[g] < 0.0f) (*mv[q])[g] = glob[q] >= 0.0 ? (float)glob[q] : 0.0f;
  if (!leq) s.eqsteps = 0;
  if (!lnumg) s.nnumg = s.eqsteps > 1000 ? s.eqsteps / 1000 : 1;
  if (!lsteps) s.mcsteps = 1;
  s.overlap_sq = s.overlap_sq * s.overlap_sq;  // gcmc.f:325 squares it
  s.minchk = std::max(1, std::min(400, s.nnumg));
}

// Peng-Robinson fugacity of guest type ig (calc_fugacity,
// utility_pack.f:1428-1500) with fluid_properties' constants
// (utility_pack.f:1364-1424).  Single-precision literals of the reference
// stay single precision (its 0.37464, sqrt(2.0), ...).  The Newton
// iteration for the compressibility factor is capped (the reference's is
// not).
static double pr_fugacity(const System &s, int ig, const std::vector<int> &kind,
                          const std::vector<std::vector<double>> &kfug) {
  const int G = s.ntpguest;
  const double R = (double)8.314f, T = s.temp;
  static const float acc[6] = {0.0f, 0.037f, 0.225f, 0.011f, 0.099f, -0.217f};
  static const float tcr[6] = {0.0f, 126.2f, 304.12f, 190.56f, 305.32f, 32.98f};
  static const float pcr[6] = {0.0f, 3.398e6f, 7.374e6f, 4.599e6f, 4.872e6f, 1.293e6f};
  std::vector<double> a(G + 1), b(G + 1);
  for (int i = 1; i <= G; ++i) {
    const double w = acc[kind[i]], tc = tcr[kind[i]], pc = pcr[kind[i]];
    const double kappa = (double)0.37464f + (double)1.54226f * w - (double)0.26992f * w * w;
    const double at = (1.0 + kappa * (1.0 - std::sqrt(T / tc)));
    const double rt = R * tc;
    a[i] = (double)0.45724f * (rt * rt) / pc * (at * at);
    b[i] = (double)0.0778f * R * tc / pc;
  }
  double asys = 0.0, bsys = 0.0;
  if (G == 1) {
    asys = a[1];
    bsys = b[1];
  } else {
    for (int i = 1; i <= G; ++i) {
      for (int j = 1; j <= G; ++j)
        asys = asys + s.gstmolfract[i] * s.gstmolfract[j] * std::sqrt(a[i] * a[j]) * (1.0 - kfug[i][j]);
      bsys = bsys + s.gstmolfract[i] * b[i];
    }
  }
  const double P = s.gstpress[ig];
  const double A = asys * P / ((R * T) * (R * T));
  const double B = bsys * P / R / T;
  const double alpha = B - 1.0, beta_f = A - 3.0 * B * B - 2.0 * B, gamma = -A * B + B * B + B * B * B;
  double z1 = 1.0, z0 = 0.0;
  for (int it = 0;; ++it) {
    if (it > 10000) raise(FMC_ERR_INPUT, "Peng-Robinson compressibility did not converge");
    z0 = z1;
    z1 = z0 - (z0 * z0 * z0 + alpha * (z0 * z0) + beta_f * z0 + gamma) /
                  (3.0 * (z0 * z0) + 2.0 * alpha * z0 + beta_f);
    if (std::fabs(z1 - z0) < 1.0e-5) break;
  }
  double sum_za = 0.0;
  for (int i = 1; i <= G; ++i)
    sum_za = sum_za + s.gstmolfract[i] * std::sqrt(a[ig] * a[i]) * (1.0 - kfug[ig][i]);
  const float r2 = std::sqrt(2.0f);
  const double two_r2 = (double)(2.0f * r2), p1 = (double)(1.0f + r2), m1 = (double)(1.0f - r2);
  const double coeff = std::exp(b[ig] / bsys * (z1 - 1.0) - std::log(z1 - B) -
                                asys / (two_r2 * bsys * R * T) * (2.0 * sum_za / asys - b[ig] / bsys) *
                                    std::log((z1 + p1 * B) / (z1 + m1 * B)));
  return coeff * s.gstmolfract[ig] * s.gstpress[ig];
}

// fugacity (utility_pack.f:1206-1310): partial pressures, mole fractions and
// (CONTROL "fugacity") Peng-Robinson fugacities; then the move-frequency
// normalisation (gcmc.f:341-386) in REAL*4.
void finish_control(System &s) {
  int G = s.ntpguest;
  // probability grid and folding cell (gcmc.f:258-306)
  for (int i = 1; i <= 9; ++i) {
    const int ci = (int)std::ceil(double(i) / 3.0);
    s.ucell[i - 1] = s.cell[i - 1] / double(s.gridfactor[ci - 1]);
  }
  invert3(s.ucell, s.rucell);
  if (s.lprob) {
    for (int d = 0; d < 3; ++d) {
      const double gd = s.celprp[d] / std::ceil(s.celprp[d] / s.gridfactor[d] / s.griddim) / s.gridfactor[d];
      s.ngrid[d] = (int)std::ceil(s.celprp[d] / (gd * s.gridfactor[d]));
    }
  }
  bool lfract = false, lpress = true;
  double fsum = 0.0, nofract = 0.0, psum = 0.0;
  for (int i = 1; i <= G; ++i) {
    if (s.gstpress[i] < 0.0) lpress = false;
    else psum += s.gstpress[i];
    if (s.gstmolfract[i] > 0.0) {
      lfract = true;
      fsum += s.gstmolfract[i];
    } else {
      nofract += 1.0;
    }
  }
  if (lfract && !lpress) {
    if (s.total_pressure < 0.0) raise(FMC_ERR_INPUT, "no total pressure (error 2314)");
    if (G == 1) {
      s.gstmolfract[1] = 1.0;
      fsum = 1.0;
    }
    if (fsum < 1.0)
      for (int i = 1; i <= G; ++i)
        if (s.gstmolfract[i] < 0) s.gstmolfract[i] = (1.0 - fsum) / nofract;
    for (int i = 1; i <= G; ++i) s.gstpress[i] = s.total_pressure * s.gstmolfract[i];
  }
  if (!lpress && !lfract && s.total_pressure > 0.0) {
    for (int i = 1; i <= G; ++i) s.gstpress[i] = s.total_pressure;
    s.total_pressure = G * s.total_pressure;
    psum = s.total_pressure;
  }
  if (s.total_pressure > 0.0 && !lfract) {
    if (psum != s.total_pressure) s.total_pressure = psum;
    for (int i = 1; i <= G; ++i) s.gstmolfract[i] = s.gstpress[i] / s.total_pressure;
  } else if (lpress && !lfract) {
    s.total_pressure = psum;
    for (int i = 1; i <= G; ++i) s.gstmolfract[i] = s.gstpress[i] / s.total_pressure;
  }
  // fluid_properties / guess_guest (utility_pack.f:1311-1424): the guest is
  // recognised by its molecular mass; an unknown guest turns the
  // Peng-Robinson branch off for every guest type
  std::vector<int> kind(G + 1, 0);
  std::vector<std::vector<double>> kfug(G + 1, std::vector<double>(G + 1, 0.0));
  bool lfuga = s.lfuga;
  if (lfuga) {
    for (int i = 1; i <= G; ++i) {
      double mass = 0.0;
      for (double w : s.mol[s.locguest[i]].wght) mass = mass + w;
      int k = 0;
      if (mass > 27.0 && mass < 29.0) k = 1;        // N2
      else if (mass > 43.0 && mass < 45.0) k = 2;   // CO2
      else if (mass > 15.5 && mass < 17.0) k = 3;   // CH4
      else if (mass > 29.0 && mass < 31.0) k = 4;   // C2H6
      else if (mass > 1.0 && mass < 3.0) k = 5;     // H2
      kind[i] = k;
      if (k == 0) lfuga = false;
    }
    if (G == 2 && ((kind[1] == 3 && kind[2] == 4) || (kind[1] == 4 && kind[2] == 3)))
      kfug[1][2] = kfug[2][1] = (double)-0.003f;
  }
  s.gstfuga.assign(G + 1, 0.0);
  for (int i = 1; i <= G; ++i) s.gstfuga[i] = lfuga ? pr_fugacity(s, i, kind, kfug) : s.gstpress[i];
  for (int i = 1; i <= G; ++i) {
    float nrm = s.mcinsf[i] + s.mcdelf[i] + s.mcdisf[i] + s.mcjmpf[i] + s.mcswpf[i] +
                s.mctraf[i] + s.mcrotf[i] + s.mcswif[i];
    if (nrm == 0.0f) {
      nrm = 1.0f;
      s.mcinsf[i] = s.mcdelf[i] = s.mcdisf[i] = (float)(1.0 / 3.0);
      s.mcjmpf[i] = s.mcswpf[i] = s.mctraf[i] = s.mcrotf[i] = s.mcswif[i] = 0.0f;
    }
    s.mcinsf[i] = s.mcinsf[i] / nrm;
    s.mcdelf[i] = s.mcinsf[i] + (s.mcdelf[i] / nrm);
    s.mcdisf[i] = s.mcdelf[i] + (s.mcdisf[i] / nrm);
    s.mcjmpf[i] = s.mcdisf[i] + (s.mcjmpf[i] / nrm);
    s.mcswpf[i] = s.mcjmpf[i] + (s.mcswpf[i] / nrm);
    s.mctraf[i] = s.mcswpf[i] + (s.mctraf[i] / nrm);
    s.mcrotf[i] = s.mctraf[i] + (s.mcrotf[i] / nrm);
    s.mcswif[i] = s.mcrotf[i] + (s.mcswif[i] / nrm);
    // swap needs a partner type; switch acts only with three or more guest
    // types (it returns without a draw unless two other types hold molecules)
    if (s.mcswpf[i] > s.mcjmpf[i] && G < 2) raise(FMC_ERR_INPUT, "swap moves need two guest types");
  }
  s.beta = 1.0 / (kKboltz * s.temp);
  s.statvolm = s.volm * 1e-30;
}

void build_derived(System &s);

// erfcgen (ewald.f:1-30), lrcorrect's per-pair tail constants
// (vdw_terms.f:548-645), then build_derived.
void build_tables(System &s) {
  const double a1 = 0.254829592, a2 = -0.284496736, a3 = 1.421413741;
  const double a4 = -1.453152027, a5 = 1.061405429, pp = 0.3275911;
  s.drewd = s.rcut / double(s.mxegrd - 4);
  s.erc.assign(s.mxegrd + 3, 0.0);
  for (int i = 1; i <= s.mxegrd; ++i) {
    double rr = double(i) * s.drewd;
    double tt = 1.0 / (1.0 + pp * s.alpha * rr);
    double ar = s.alpha * rr;
    double ex = std::exp(-(ar * ar));
    s.erc[i] = tt * (a1 + tt * (a2 + tt * (a3 + tt * (a4 + tt * a5)))) * ex / rr;
  }
  // tail constants per unique type pair
  int npair = s.ntpatm * (s.ntpatm + 1) / 2;
  s.steadd.assign(npair + 1, 0.0);
  int iv = 0;
  for (int i = 1; i <= s.ntpatm; ++i)
    for (int j = 1; j <= i; ++j) {
      ++iv;
      int k = s.lstvdw[iv];
      double e = 0.0;
      if (s.ltpvdw[k] == 1) {
        e = s.prmvdw[k][1] / (9.0 * std::pow(s.rcut, 9)) - s.prmvdw[k][2] / (3.0 * std::pow(s.rcut, 3));
      } else if (s.ltpvdw[k] == 2) {
        double ep = s.prmvdw[k][1], sg = s.prmvdw[k][2];
        e = 4.0 * ep * (std::pow(sg, 12) / (9.0 * std::pow(s.rcut, 9)) -
                        std::pow(sg, 6) / (3.0 * std::pow(s.rcut, 3)));
      }
      if (i != j) e *= 2.0;
      s.steadd[iv] = e;
    }
  build_derived(s);
}

// Framework type counts, k-vector list (ewald.f:151-315) and
// excluding_ewald_charges (gcmc.f:2662-2761): what follows from the cell,
// the molecules and the Ewald parameters alone.
void build_derived(System &s) {
  const double a1 = 0.254829592, a2 = -0.284496736, a3 = 1.421413741;
  const double a4 = -1.453152027, a5 = 1.061405429, pp = 0.3275911;
  const MolType &fw = s.mol[s.fw_mol];
  s.n_fw = fw.nummols * fw.natoms;
  s.numtyp_fw.assign(s.ntpatm + 1, 0);
  s.numfrz_fw.assign(s.ntpatm + 1, 0);
  for (int a = 0; a < fw.natoms; ++a) {
    s.numtyp_fw[fw.ltp[a]] += fw.nummols;
    if (fw.frz[a]) s.numfrz_fw[fw.ltp[a]] += fw.nummols;
  }
  // k vectors in the half space, reference loop order
  s.kl.clear();
  s.km.clear();
  s.kn.clear();
  s.rksq.clear();
  s.akk.clear();
  double det[10];
  cell_props(s.rcell, det);
  double twopi = 2.0 * kPi;
  double rcp = std::min(double(s.kmax[0]) * det[6],
                        std::min(double(s.kmax[1]) * det[7], double(s.kmax[2]) * det[8]));
  rcp = rcp * 1.05 * twopi;
  double rcp2 = rcp * rcp;
  double ralph = -0.25 / (s.alpha * s.alpha);
  int mmin = 0, nmin = 1;
  const double *rc = s.rcell;
  for (int ll = 0; ll <= s.kmax[0]; ++ll) {
    double t1 = twopi * double(ll);
    double x1 = t1 * rc[0], y1 = t1 * rc[3], z1 = t1 * rc[6];
    for (int mm = mmin; mm <= s.kmax[1]; ++mm) {
      double t2 = twopi * double(mm);
      double x2 = x1 + t2 * rc[1], y2 = y1 + t2 * rc[4], z2 = z1 + t2 * rc[7];
      for (int nn = nmin; nn <= s.kmax[2]; ++nn) {
        double t3 = twopi * double(nn);
        double x3 = x2 + t3 * rc[2], y3 = y2 + t3 * rc[5], z3 = z2 + t3 * rc[8];
        double k2 = x3 * x3 + y3 * y3 + z3 * z3;
        if (k2 <= rcp2) {
          s.kl.push_back(ll);
          s.km.push_back(mm);
          s.kn.push_back(nn);
          s.rksq.push_back(k2);
          s.akk.push_back(std::exp(ralph * k2) * (1.0 / k2));
        }
      }
      nmin = -s.kmax[2];
    }
    mmin = -s.kmax[1];
  }
  s.newld = (int)s.kl.size();
  // ewald3 for each guest type (ewald.f:735-790)
  s.ewald3en.assign(s.maxmls + 1, 0.0);
  for (int g = 1; g <= s.ntpguest; ++g) {
    int m = s.locguest[g];
    const MolType &gm = s.mol[m];
    const auto &t = s.guest_tmpl[g];
    double e3 = 0.0;
    for (int i = 0; i < gm.natoms - 1; ++i) {
      double chgea = gm.chg[i] / s.epsq * kR4pie0;
      double e = 0.0;
      for (int j = i + 1; j < gm.natoms; ++j) {
        double dx = t[3 * i] - t[3 * j], dy = t[3 * i + 1] - t[3 * j + 1],
               dz = t[3 * i + 2] - t[3 * j + 2];
        min_image(s, dx, dy, dz);
        double chgprd = chgea * gm.chg[j];
        double rr = std::sqrt(dx * dx + dy * dy + dz * dz);
        double alpr = rr * s.alpha, alpr2 = alpr * alpr, erfr;
        if (alpr < 1.0e-2) {
          erfr = 2.0 * chgprd * (s.alpha / kSqrPi) *
                 (1.0 + alpr2 * (-0.333333333333 +
                                 alpr2 * (0.1 + alpr2 * (-0.02380952381 + alpr2 * 4.62962962963e-3))));
        } else {
          double tt = 1.0 / (1.0 + pp * s.alpha * rr);
          double ex = std::exp(-(alpr * alpr));
          erfr = (1.0 - tt * (a1 + tt * (a2 + tt * (a3 + tt * (a4 + tt * a5)))) * ex) * chgprd / rr;
        }
        e += erfr;
      }
      e3 += e;
    }
    s.ewald3en[m] = e3;
  }
}

}  // namespace

// The system from a host's start-up arrays (fmc_upload_system): the fields
// fmc_system_load fills from the input files, taken from the descriptor,
// then the parts that follow from them (build_derived).
void upload_system(const fmc_system_desc &d, System &s) {
  auto need = [](bool ok, const char *what) {
    if (!ok) raise(FMC_ERR_ARG, std::string("fmc_upload_system: ") + what);
  };
  need(d.imcon >= 1 && d.imcon <= 3, "imcon must be 1, 2 or 3");
  need(d.maxmls >= 2 && d.maxmls <= FMC_MAX_MOLTYPES, "maxmls out of range");
  need(d.ntpguest >= 1 && d.ntpguest <= FMC_MAX_GUEST_TYPES, "ntpguest out of range");
  need(d.ntpatm >= 1 && d.ntpatm <= 16, "ntpatm out of range");
  need(d.mxegrd >= 8 && d.ntpvdw >= 1, "table sizes out of range");
  need(d.erc && d.vvv && d.ltpvdw && d.prmvdw && d.lstvdw && d.steadd, "null table");
  need(d.numatoms && d.nummols && d.is_guest && d.ltype && d.charge && d.mass && d.frozen,
       "null molecule array");
  need(d.guest_tmpl && d.fugacity && d.delr && d.disp_ratio && d.tran_ratio && d.rota_ratio &&
           d.move_freq, "null guest array");
  need(d.rcut > 0.0 && d.alpha > 0.0 && d.temp > 0.0 && d.engunit > 0.0 && d.epsq > 0.0,
       "non-positive rcut, alpha, temperature, engunit or epsq");
  need(d.drewd > 0.0 && d.dlrpot > 0.0, "non-positive table spacing");
  for (int i = 0; i < 3; ++i) need(d.kmax[i] >= 1, "kmax below 1");
  s = System();
  s.imcon = d.imcon;
  for (int i = 0; i < 9; ++i) s.cell[i] = d.cell[i];
  cell_props(s.cell, s.celprp);
  s.volm = s.celprp[9];
  need(s.volm > 0.0, "cell has no volume");
  invert3(s.cell, s.rcell);
  if (s.imcon == 2 || s.imcon == 1)
    for (int i : {1, 2, 3, 5, 6, 7})
      if (std::fabs(s.cell[i]) > 1e-10) raise(FMC_ERR_INPUT, "cell is not orthorhombic (error 410)");
  s.engunit = d.engunit;
  s.temp = d.temp;
  s.rcut = s.rvdw = d.rcut;
  s.alpha = d.alpha;
  s.epsq = s.eps = d.epsq;
  for (int i = 0; i < 3; ++i) s.kmax[i] = d.kmax[i];
  s.overlap_sq = d.overlap * d.overlap;
  s.surftol = d.surftol;
  s.eqsteps = d.eqsteps;
  s.nwindsteps = std::max(1, d.nwindsteps);
  s.minchk = std::max(1, d.minchk);
  s.laccsample = d.laccsample != 0;
  // tables, 1-based as the reference keeps them
  s.ntpatm = d.ntpatm;
  s.mxatyp = d.ntpatm;
  s.mxegrd = d.mxegrd;
  s.drewd = d.drewd;
  s.dlrpot = d.dlrpot;
  s.erc.assign(s.mxegrd + 3, 0.0);
  for (int i = 1; i <= s.mxegrd; ++i) s.erc[i] = d.erc[i - 1];
  const int npair = s.ntpatm * (s.ntpatm + 1) / 2;
  s.ntpvdw = d.ntpvdw;
  s.maxvdw = std::max(s.ntpvdw, npair);
  s.ltpvdw.assign(s.maxvdw + 2, -1);
  s.lstvdw.assign(s.maxvdw + 2, 0);
  s.prmvdw.assign(s.maxvdw + 2, std::array<double, 6>{0, 0, 0, 0, 0, 0});
  s.vvv.assign(s.maxvdw + 2, std::vector<double>(s.mxegrd + 3, 0.0));
  for (int k = 1; k <= s.ntpvdw; ++k) {
    need(d.ltpvdw[k - 1] == 1 || d.ltpvdw[k - 1] == 2, "ltpvdw: only 12-6 (1) and lj (2) are supported");
    s.ltpvdw[k] = d.ltpvdw[k - 1];
    s.prmvdw[k][1] = d.prmvdw[k - 1];
    s.prmvdw[k][2] = d.prmvdw[s.ntpvdw + k - 1];
    for (int i = 1; i <= s.mxegrd; ++i) s.vvv[k][i] = d.vvv[(size_t)(k - 1) * s.mxegrd + (i - 1)];
  }
  s.steadd.assign(npair + 1, 0.0);
  for (int p = 1; p <= npair; ++p) {
    need(d.lstvdw[p - 1] >= 1 && d.lstvdw[p - 1] <= s.ntpvdw + 1, "lstvdw entry out of range");
    s.lstvdw[p] = d.lstvdw[p - 1];
    s.steadd[p] = d.steadd[p - 1];
  }
  // molecule types
  s.maxmls = d.maxmls;
  s.mol.assign(s.maxmls + 1, MolType());
  s.locguest.assign(1, 0);
  s.locfram.assign(1, 0);
  s.guest_tmpl.assign(1, {});
  s.unqatm.assign(s.ntpatm + 1, "");
  size_t site = 0, fwxyz = 0, tmpl = 0;
  for (int m = 1; m <= s.maxmls; ++m) {
    MolType &mt = s.mol[m];
    mt.natoms = d.numatoms[m - 1];
    mt.nummols = d.nummols[m - 1];
    mt.guest = d.is_guest[m - 1] != 0;
    need(mt.natoms >= 1 && mt.nummols >= 0, "molecule sizes out of range");
    mt.site.assign(mt.natoms, "");
    mt.wght.assign(mt.natoms, 0.0);
    mt.chg.assign(mt.natoms, 0.0);
    mt.frz.assign(mt.natoms, 0);
    mt.ltp.assign(mt.natoms, 0);
    for (int a = 0; a < mt.natoms; ++a, ++site) {
      mt.ltp[a] = d.ltype[site];
      need(mt.ltp[a] >= 1 && mt.ltp[a] <= s.ntpatm, "ltype out of range");
      mt.chg[a] = d.charge[site];
      mt.wght[a] = d.mass[site];
      mt.frz[a] = d.frozen[site] ? 1 : 0;
    }
    if (mt.guest) {
      need(mt.nummols == 0, "guests are created on the device (nummols of a guest type must be 0)");
      need(mt.natoms <= FMC_MAX_SITES, "guest has too many sites");
      s.locguest.push_back(m);
      ++s.ntpguest;
      s.guest_tmpl.push_back(std::vector<double>(d.guest_tmpl + tmpl, d.guest_tmpl + tmpl + 3 * mt.natoms));
      tmpl += 3 * mt.natoms;
    } else {
      s.locfram.push_back(m);
      ++s.ntpfram;
      need(d.fw_xyz != nullptr, "null framework coordinates");
      const size_t n = 3 * (size_t)mt.nummols * mt.natoms;
      mt.xyz.assign(d.fw_xyz + fwxyz, d.fw_xyz + fwxyz + n);
      fwxyz += n;
      for (int a = 0; a < mt.natoms; ++a)
        if (!mt.frz[a]) raise(FMC_ERR_INPUT, "non-frozen framework atoms are not supported");
    }
  }
  if (s.ntpfram != 1) raise(FMC_ERR_INPUT, "exactly one framework molecule type is supported");
  need(s.ntpguest == d.ntpguest, "ntpguest differs from the guest molecule types");
  s.fw_mol = s.locfram[1];
  s.sumchg = 0.0;
  for (int it = 1; it <= s.maxmls; ++it)
    for (int l = 0; l < s.mol[it].natoms; ++l) s.sumchg += double(s.mol[it].nummols) * s.mol[it].chg[l];
  // run control per guest type
  const int G = s.ntpguest;
  s.gstfuga.assign(G + 1, 0.0);
  s.gstpress.assign(G + 1, 0.0);
  s.gstmolfract.assign(G + 1, 0.0);
  s.delr.assign(G + 1, 0.0);
  s.disp_ratio.assign(G + 1, 0.0);
  s.tran_ratio.assign(G + 1, 0.0);
  s.rota_ratio.assign(G + 1, 0.0);
  s.guest_insert.assign(G + 1, 0);
  for (auto *v : {&s.mcinsf, &s.mcdelf, &s.mcdisf, &s.mcjmpf, &s.mcswpf, &s.mctraf, &s.mcrotf, &s.mcswif})
    v->assign(G + 1, 0.0f);
  s.nprob.assign(G + 1, 0);
  s.lprobeng.assign(G + 1, 0);
  for (int g = 1; g <= G; ++g) {
    s.gstfuga[g] = s.gstpress[g] = d.fugacity[g - 1];
    s.delr[g] = d.delr[g - 1];
    s.disp_ratio[g] = d.disp_ratio[g - 1];
    s.tran_ratio[g] = d.tran_ratio[g - 1];
    s.rota_ratio[g] = d.rota_ratio[g - 1];
    s.guest_insert[g] = d.create ? d.create[g - 1] : 0;
    const float *f = d.move_freq + 8 * (g - 1);
    s.mcinsf[g] = f[0];
    s.mcdelf[g] = f[1];
    s.mcdisf[g] = f[2];
    s.mcjmpf[g] = f[3];
    s.mcswpf[g] = f[4];
    s.mctraf[g] = f[5];
    s.mcrotf[g] = f[6];
    s.mcswif[g] = f[7];
    for (int k = 1; k < 8; ++k) need(f[k] >= f[k - 1], "move thresholds must be cumulative");
    if (s.mcswpf[g] > s.mcjmpf[g] && G < 2) raise(FMC_ERR_INPUT, "swap moves need two guest types");
  }
  for (int i = 0; i < 9; ++i) s.ucell[i] = s.cell[i];  // no probability grids
  invert3(s.ucell, s.rucell);
  s.beta = 1.0 / (kKboltz * s.temp);
  s.statvolm = s.volm * 1e-30;
  build_derived(s);
  if (s.newld != d.newld)
    raise(FMC_ERR_INPUT, "fmc_upload_system: the host's newld (" + std::to_string(d.newld) +
                             ") differs from the k-vectors of cell, kmax and alpha (" +
                             std::to_string(s.newld) + ")");
}

void load_system(const std::string &dir, System &s) {
  scan_inputs(dir, s);
  read_field(dir, s);
  read_config(dir, s);
  read_control(dir, s);
  finish_control(s);
  build_tables(s);
}

}  // namespace fmc

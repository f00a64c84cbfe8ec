// fmc_internal.h -- host-side system description shared by the set-up code
// and the CUDA launch code.  Not part of the public ABI.
#pragma once

#include <array>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/fastmc_gb300.h"

namespace fmc {

// Physical constants of the reference (utility_pack.f:101-147).
constexpr double kPi = 3.141592653589793;
constexpr double kSqrPi = 1.7724538509055159;
constexpr double kR4pie0 = 138935.4835;
constexpr double kKboltz = 1.9872041e-3;
constexpr double kBoltz = 1.3806503e-23;
constexpr double kRgas = 8.314472 / 4184.0;
constexpr double kMinAngle = kPi / 18.0;
constexpr double kDelrMin = 0.1;

struct MolType {
  std::string name;
  bool guest = false;
  int nummols = 0;
  int natoms = 0;
  std::vector<std::string> site;   // 0-based sites
  std::vector<double> wght, chg;
  std::vector<int> frz, ltp;       // ltp: 1-based unique atom type
  std::vector<double> xyz;         // nummols*natoms*3 coordinates (CONFIG)
};

// Everything the reference computes at start-up that the energy path needs.
struct System {
  int imcon = 0;
  double cell[9] = {0}, rcell[9] = {0}, celprp[10] = {0};
  double volm = 0, statvolm = 0, engunit = 1.0, sumchg = 0;
  int maxmls = 0, ntpguest = 0, ntpfram = 0, ntpatm = 0, mxatyp = 0;
  int ntpvdw = 0, maxvdw = 0;
  std::vector<MolType> mol;              // 1-based (mol[0] unused)
  std::vector<int> locguest, locfram;    // 1-based
  std::vector<std::string> unqatm;       // 1-based
  std::vector<std::vector<double>> guest_tmpl;  // [iguest] natoms*3, centred
  // van der Waals (vdw_module.f)
  int mxegrd = 0;
  double dlrpot = 0, drewd = 0;
  std::vector<int> ltpvdw, lstvdw;                 // 1-based
  std::vector<std::array<double, 6>> prmvdw;       // [ivdw][1..5]
  std::vector<std::vector<double>> vvv;            // [ivdw][1..mxegrd+2]
  std::vector<double> erc;                         // [1..mxegrd+2]
  std::vector<double> steadd;                      // [loc2 pair]
  // framework type counts (lrcorrect)
  std::vector<int> numtyp_fw, numfrz_fw;           // [atype]
  // control
  double temp = 0, rcut = 0, rvdw = 0, initdelr = 0, alpha = 0, eps = 0;
  // overlap distance (default 1.5 A, gcmc.f:153); squared after CONTROL
  double overlap_sq = 1.5, surftol = 0.0, beta = 0, epsq = 1.0;
  int kmax[3] = {0, 0, 0};
  int mcsteps = 1, eqsteps = 0, nwind = 1, nwindsteps = 1, nnumg = 1;
  int minchk = 1;
  bool laccsample = false;
  double total_pressure = -1.0;
  bool lfuga = false;  // CONTROL "fugacity": Peng-Robinson fugacities
  std::vector<double> gstpress, gstmolfract, gstfuga, delr;  // [iguest]
  std::vector<double> disp_ratio, tran_ratio, rota_ratio;
  std::vector<float> mcinsf, mcdelf, mcdisf, mcjmpf, mcswpf, mctraf, mcrotf,
      mcswif;
  std::vector<int> guest_insert;
  // probability grids (storeprob, gcmc.f:258-306): CONTROL "probability"
  // blocks, "grid spacing", "grid factor"
  bool lprob = false;
  int ntprob = 0;
  double griddim = 0.1;
  int gridfactor[3] = {1, 1, 1};
  int ngrid[3] = {0, 0, 0};
  double ucell[9] = {0}, rucell[9] = {0};
  std::vector<int> nprob, lprobeng;              // [iguest]
  std::vector<int> nprobsites;                   // [1..ntprob]
  std::vector<std::vector<int>> lprobsites;      // [1..ntprob][1..]
  // k vectors in the reference order (ewald.f:151-315)
  int newld = 0;
  std::vector<int> kl, km, kn;
  std::vector<double> akk, rksq;
  // constants of the energy expressions
  std::vector<double> ewald3en;  // [mol]
  int fw_mol = 0;                // the single framework molecule type
  int n_fw = 0;                  // framework atoms
  std::string cfgname = std::string(80, ' ');  // CONFIG title (REVCON's first record)
};

// host_setup.cpp
void load_system(const std::string &dir, System &s);
void upload_system(const fmc_system_desc &d, System &s);
inline int loc2(int i, int j) {
  int a = i > j ? i : j, b = i > j ? j : i;
  return (a * (a - 1)) / 2 + b;
}

void set_error(const std::string &msg);
struct Error {
  int code;
  std::string msg;
};
[[noreturn]] void raise(int code, const std::string &msg);

}  // namespace fmc

struct fmc_system {
  fmc::System s;
};

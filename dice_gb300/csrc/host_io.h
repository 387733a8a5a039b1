// Host-side integrals, heat-bath tables and input schedule.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "status.h"

namespace shci {

struct HostInts {
  int norb = 0, nelec = 0;
  double coreE = 0.0, maxEntry = 0.0;
  std::vector<double> I1;  // (2n)x(2n) spin-orbital
  std::vector<double> I2;  // 8-fold packed spatial
  std::vector<double> Direct, Exchange;
  double i2(int i, int j, int k, int l) const;  // spin-orbital accessor
};

struct HostHeatBath {
  std::vector<float> sameVal, oppVal;
  std::vector<int16_t> samePairs, oppPairs;
  std::vector<int64_t> sameStart, oppStart;
  std::vector<double> singles;
};

struct Restriction {
  int minElec = 0, maxElec = 10000;
  uint64_t mask = 0;  // spatial orbitals
};

// Variational and deterministic-PT subset of the reference's schedule
// (SHCI/input.h:35-194).
struct Schedule {
  std::vector<std::vector<int>> occupied;
  std::vector<double> epsilon1;
  int nroots = 1;
  double davidsonTol = 5e-5, davidsonTolLoose = 5e-5, dE = 1e-8;
  bool direct = false;
  int ncore = 0, nact = 1000000;
  std::vector<Restriction> restrictions;
  std::string integralFile = "FCIDUMP";
  int mode = -1;       // precision keyword: -1 unset, 0 fp64, 1 mixed
  bool block = false;  // blockdavidson keyword
  int precond = -1;    // precond keyword: -1 unset, 0 plain, 1 pt2, 2 mlp
  int basis_max = 0, basis_keep = 0;  // davidsonBasis keyword: 0 = the reference's subspace
  double epsilon2 = 1.e-8;  // PT threshold (SHCI/input.cpp:58)
  bool stochastic = true;   // `deterministic` clears it (SHCI/input.cpp:322-323)
  // semistochastic PT (SHCI/input.cpp:59-86): threshold of its deterministic
  // part, draws per iteration (-1: not set), iteration cap, target error,
  // seed (-1: not set; the reference then seeds from the clock)
  double epsilon2Large = 1000.0;
  int sampleN = -1;
  int nPTiter = 1000000;
  double targetError = 1.e-4;
  long long seed = -1;
  int writeBest = 0;  // writebestdeterminants (SHCI/input.cpp:243-244)
  // time-reversal symmetry (Treversal, SHCI/input.cpp:253-258): 0 off, +1 or
  // -1 the sign that relates a determinant's coefficient to its alpha <-> beta
  // flipped partner's
  int trev = 0;
  // checkpoints (SHCI/input.cpp:72, 176-183, 330-331, 400): io writes the
  // variational result after every iteration (default), noio does not;
  // restart = 1 resumes after the saved iteration, 2 (fullrestart) reruns the
  // schedule from the saved space; prefix is the checkpoint directory (a
  // relative prefix is taken relative to baseDir, the input file's directory)
  bool io = true;
  int restart = 0;
  std::string prefix = ".";
  std::string baseDir = ".";
};

void split_tokens(const std::string& in, const char* delims, std::vector<std::string>& tok);
bool iequal(const std::string& a, const std::string& b);
void read_fcidump(const std::string& path, HostInts& H);
void build_heatbath(const HostInts& H, HostHeatBath& hb);
void read_input(const std::string& path, Schedule& s);

}  // namespace shci

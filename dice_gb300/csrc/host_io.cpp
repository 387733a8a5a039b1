// Host-side input handling of the engine:
//   * FCIDUMP reader with the reference's parse rules (readIntegrals,
//     SHCI/integral.cpp:43-225);
//   * heat-bath tables: per spatial pair (i >= j) the opposite-spin list of
//     (ia|jb) and the same-spin list of (ia|jb)-(ib|ja) (a >= b), |v| > 1e-10,
//     cast to FP32 and ordered by |FP32 value| descending, ties in reverse
//     (a, b) order -- the order in which the reference reads its compAbs
//     multimaps backwards (SHCI/integral.h:125-153, SHCI/integral.cpp:320-369);
//     and the single-excitation bound Singles(i,a) (SHCI/integral.h:143-151);
//   * the variational subset of the input.dat keyword parser
//     (SHCI/input.cpp:35-404).
#include "host_io.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

namespace shci {

// boost::trim followed by boost::split(..., is_any_of(delims), token_compress_on)
void split_tokens(const std::string& in, const char* delims, std::vector<std::string>& tok) {
  size_t b = 0, e = in.size();
  while (b < e && std::isspace((unsigned char)in[b])) ++b;
  while (e > b && std::isspace((unsigned char)in[e - 1])) --e;
  tok.clear();
  std::string cur;
  bool prev_delim = false;
  for (size_t i = b; i < e; ++i) {
    if (std::strchr(delims, in[i])) {
      if (!prev_delim) {
        tok.push_back(cur);
        cur.clear();
      }
      prev_delim = true;
    } else {
      cur.push_back(in[i]);
      prev_delim = false;
    }
  }
  tok.push_back(cur);
}

bool iequal(const std::string& a, const std::string& b) {
  if (a.size() != b.size()) return false;
  for (size_t i = 0; i < a.size(); ++i)
    if (std::tolower((unsigned char)a[i]) != std::tolower((unsigned char)b[i])) return false;
  return true;
}

static inline size_t packed_index(int i, int j, int k, int l) {
  size_t ij = (size_t)std::max(i, j) * (std::max(i, j) + 1) / 2 + std::min(i, j);
  size_t kl = (size_t)std::max(k, l) * (std::max(k, l) + 1) / 2 + std::min(k, l);
  size_t A = std::max(ij, kl), B = std::min(ij, kl);
  return A * (A + 1) / 2 + B;
}

double HostInts::i2(int i, int j, int k, int l) const {
  if (((i ^ j) & 1) || ((k ^ l) & 1)) return 0.0;
  return I2[packed_index(i >> 1, j >> 1, k >> 1, l >> 1)];
}

void read_fcidump(const std::string& path, HostInts& H) {
  std::ifstream dump(path.c_str());
  if (!dump.good()) throw Error(kErrIO, "Integral file " + path + " does not exist!");
  int norbs = -1, nelec = -1;
  std::vector<std::string> tok;
  std::string line;
  bool have_end = false;
  while (std::getline(dump, line)) {
    split_tokens(line, ", \t=", tok);
    if (tok.size() == 1 && (iequal(tok[0], "&END") || iequal(tok[0], "/"))) {
      have_end = true;
      break;
    }
    if (iequal(tok[0].substr(0, 4), "&FCI")) {
      if (tok.size() > 2 && iequal(tok[1].substr(0, 4), "NORB")) norbs = std::atoi(tok[2].c_str());
      if (tok.size() > 4 && iequal(tok[3].substr(0, 5), "NELEC")) nelec = std::atoi(tok[4].c_str());
    } else if (iequal(tok[0].substr(0, 4), "KSYM")) {
      throw Error(kErrInvalid, "KSYM (complex k-point) integrals are not supported");
    }
  }
  if (!have_end) throw Error(kErrInvalid, "FCIDUMP header has no &END line");
  if (norbs == -1 || nelec == -1) throw Error(kErrInvalid, "could not read the norbs or nelec");
  if (norbs < 1 || norbs > kMaxOrbitals) throw Error(kErrInvalid, "NORB must be in 1..64");
  if (nelec < 0 || nelec > 2 * norbs) throw Error(kErrInvalid, "NELEC out of range");
  H.norb = norbs;
  H.nelec = nelec;
  const size_t npair = (size_t)norbs * (norbs + 1) / 2;
  H.I2.assign(npair * (npair + 1) / 2, 0.0);
  const int n2 = 2 * norbs;
  H.I1.assign((size_t)n2 * n2, 0.0);
  H.coreE = 0.0;
  size_t nlines = 0;
  while (std::getline(dump, line)) {
    split_tokens(line, ", \t", tok);
    if (tok.size() != 5) continue;
    char* endp = nullptr;
    double v = std::strtod(tok[0].c_str(), &endp);
    int a = std::atoi(tok[1].c_str()), b = std::atoi(tok[2].c_str()), c = std::atoi(tok[3].c_str()),
        d = std::atoi(tok[4].c_str());
    ++nlines;
    if (a == 0 && b == 0 && c == 0 && d == 0) {
      H.coreE = v;
    } else if (b == 0 && c == 0 && d == 0) {
      continue;  // orbital energy
    } else if (c == 0 && d == 0) {
      if (a < 1 || b < 1 || a > norbs || b > norbs) throw Error(kErrInvalid, "one-electron index out of range: " + line);
      H.I1[(size_t)(2 * (a - 1)) * n2 + 2 * (b - 1)] = v;
      H.I1[(size_t)(2 * (a - 1) + 1) * n2 + 2 * (b - 1) + 1] = v;
      H.I1[(size_t)(2 * (b - 1)) * n2 + 2 * (a - 1)] = v;
      H.I1[(size_t)(2 * (b - 1) + 1) * n2 + 2 * (a - 1) + 1] = v;
    } else {
      if (a < 1 || b < 1 || c < 1 || d < 1 || a > norbs || b > norbs || c > norbs || d > norbs)
        throw Error(kErrInvalid, "two-electron index out of range: " + line);
      H.I2[packed_index(a - 1, b - 1, c - 1, d - 1)] = v;
    }
  }
  if (nlines == 0) throw Error(kErrInvalid, "FCIDUMP has no integral lines");
  double best = H.I2.empty() ? 0.0 : H.I2[0];
  for (double v : H.I2)
    if (std::fabs(best) < std::fabs(v)) best = v;
  H.maxEntry = best;
  H.Direct.assign((size_t)norbs * norbs, 0.0);
  H.Exchange.assign((size_t)norbs * norbs, 0.0);
  for (int i = 0; i < norbs; i++)
    for (int j = 0; j < norbs; j++) {
      H.Direct[(size_t)i * norbs + j] = H.I2[packed_index(i, i, j, j)];
      H.Exchange[(size_t)i * norbs + j] = H.I2[packed_index(i, j, j, i)];
    }
}

namespace {
struct Entry {
  float v;
  int16_t a, b;
  int32_t seq;
};
void emit_sorted(std::vector<Entry>& e, std::vector<float>& vals, std::vector<int16_t>& pairs) {
  std::sort(e.begin(), e.end(), [](const Entry& x, const Entry& y) {
    float ax = std::fabs(x.v), ay = std::fabs(y.v);
    if (ax != ay) return ax > ay;
    return x.seq > y.seq;
  });
  for (const Entry& x : e) {
    vals.push_back(x.v);
    pairs.push_back(x.a);
    pairs.push_back(x.b);
  }
}
}  // namespace

void build_heatbath(const HostInts& H, HostHeatBath& hb) {
  const int n = H.norb;
  const double thr = 1.e-10;
  hb.sameVal.clear();
  hb.oppVal.clear();
  hb.samePairs.clear();
  hb.oppPairs.clear();
  hb.sameStart.assign(1, 0);
  hb.oppStart.assign(1, 0);
  std::vector<Entry> same, opp;
  same.reserve((size_t)n * n);
  opp.reserve((size_t)n * n);
  for (int i = 0; i < n; i++)
    for (int j = 0; j <= i; j++) {
      same.clear();
      opp.clear();
      int32_t ss = 0, so = 0;
      for (int a = 0; a < n; a++)
        for (int b = 0; b < n; b++) {
          const double iajb = H.I2[packed_index(i, a, j, b)];
          if (std::fabs(iajb) > thr) opp.push_back({(float)iajb, (int16_t)a, (int16_t)b, so++});
          if (a >= b) {
            const double s = iajb - H.I2[packed_index(i, b, j, a)];
            if (std::fabs(s) > thr) same.push_back({(float)s, (int16_t)a, (int16_t)b, ss++});
          }
        }
      emit_sorted(same, hb.sameVal, hb.samePairs);
      emit_sorted(opp, hb.oppVal, hb.oppPairs);
      hb.sameStart.push_back((int64_t)hb.sameVal.size());
      hb.oppStart.push_back((int64_t)hb.oppVal.size());
    }
  const int n2 = 2 * n;
  hb.singles.assign((size_t)n2 * n2, 0.0);
  for (int i = 0; i < n2; i++)
    for (int a = 0; a < n2; a++) {
      double s = std::fabs(H.I1[(size_t)i * n2 + a]);
      for (int j = 0; j < n2; j++) {
        double t = H.i2(i, a, j, j) - H.i2(i, j, j, a);
        if (std::fabs(s) < std::fabs(t)) s = std::fabs(t);
      }
      hb.singles[(size_t)i * n2 + a] = s;
    }
}

// Keywords accepted and ignored: they configure stages outside the
// variational loop (RDM variants, printing, SOC, cdfci, time reversal).
static const char* kIgnored[] = {
    "printbestdeterminants", "printalldeterminants", "dordm", "DoOneRDM",
    "DoSpinOneRDM", "dospinrdm", "TransitionRDM", "DoThreeRDM", "DoFourRDM", "outputlevel",
    "num_thrds", "nblocks", "excitation", "nvirt", "extrapolate", "relaxedRDM", "quasiq", "dosoc",
    "dosocqdpt", "dogtensor", "socmultiplier", "doresponse", "onlyperturbative", "algorithm", "dolcc",
    "pointGroup", "spin", "irrep", "searchForLowestEnergyDet", "cdfciTol", "cdfciIter", "cdfciOn",
    "reportInterval", "z_threshold", "cdfciSample", "eps", "maxseniority", "maxexcitation", "SenioAndExc",
    "diskdavidson"};

void read_input(const std::string& path, Schedule& s) {
  std::ifstream ifs(path.c_str());
  if (!ifs.good()) throw Error(kErrIO, "cannot open input file " + path);
  std::stringstream dump;
  dump << ifs.rdbuf();
  int maxiter = -1, nocc = -1;
  std::vector<int> sweep_iter;
  std::vector<double> sweep_eps;
  std::vector<std::string> tok;
  std::string line;
  while (std::getline(dump, line)) {
    split_tokens(line, ", \t\n", tok);
    const std::string& arg = tok[0];
    if (arg.empty() || arg[0] == '#') continue;
    auto need = [&](size_t k) {
      if (tok.size() <= k) throw Error(kErrInvalid, "keyword " + arg + " needs a value");
    };
    if (iequal(arg, "nocc")) {
      need(1);
      nocc = std::atoi(tok[1].c_str());
      std::vector<std::string> t2;
      while (true) {
        if (!std::getline(dump, line)) throw Error(kErrInvalid, "nocc block has no end");
        split_tokens(line, ", \t", t2);
        if (iequal(t2[0], "end")) break;
        if ((int)t2.size() != nocc)
          throw Error(kErrInvalid, "nocc: " + std::to_string(nocc) + " neq " + std::to_string(t2.size()));
        std::vector<int> occ;
        for (auto& x : t2) occ.push_back(std::atoi(x.c_str()));
        s.occupied.push_back(occ);
      }
    } else if (iequal(arg, "nact")) {
      need(1);
      s.nact = std::atoi(tok[1].c_str());
    } else if (iequal(arg, "ncore")) {
      need(1);
      s.ncore = std::atoi(tok[1].c_str());
    } else if (iequal(arg, "directdavidson")) {
      s.direct = true;
    } else if (iequal(arg, "nroots")) {
      need(1);
      s.nroots = (int)std::atof(tok[1].c_str());
    } else if (iequal(arg, "orbitals")) {
      need(1);
      s.integralFile = tok[1];
    } else if (iequal(arg, "davidsonTol")) {
      need(1);
      s.davidsonTol = std::atof(tok[1].c_str());
    } else if (iequal(arg, "davidsonTolLoose")) {
      need(1);
      s.davidsonTolLoose = std::atof(tok[1].c_str());
    } else if (iequal(arg, "dE")) {
      need(1);
      s.dE = std::atof(tok[1].c_str());
    } else if (iequal(arg, "maxiter")) {
      need(1);
      maxiter = std::atoi(tok[1].c_str());
    } else if (iequal(arg, "restrict") || iequal(arg, "restrictv")) {
      need(3);
      Restriction r;
      r.minElec = std::atoi(tok[1].c_str());
      r.maxElec = std::atoi(tok[2].c_str());
      r.mask = 0;
      for (size_t i = 3; i < tok.size(); i++) {
        int o = std::atoi(tok[i].c_str());
        if (o < 0 || o >= kMaxOrbitals) throw Error(kErrInvalid, "restriction orbital out of range");
        r.mask |= 1ull << o;
      }
      s.restrictions.push_back(r);
    } else if (iequal(arg, "schedule")) {
      std::vector<std::string> st;
      while (true) {
        if (!std::getline(dump, line)) throw Error(kErrInvalid, "schedule block has no end");
        split_tokens(line, " \t", st);
        if (iequal(st[0], "END")) break;
        if (st[0].empty() || st[0][0] == '#') continue;
        if (st.size() < 2) throw Error(kErrInvalid, "schedule line needs iteration and eps1");
        sweep_iter.push_back(std::atoi(st[0].c_str()));
        sweep_eps.push_back(std::atof(st[1].c_str()));
      }
    } else if (iequal(arg, "precision")) {
      need(1);
      if (iequal(tok[1], "fp64"))
        s.mode = 0;
      else if (iequal(tok[1], "mixed"))
        s.mode = 1;
      else
        throw Error(kErrInvalid, "precision must be fp64 or mixed");
    } else if (iequal(arg, "epsilon2")) {
      need(1);
      s.epsilon2 = std::atof(tok[1].c_str());
    } else if (iequal(arg, "deterministic")) {
      s.stochastic = false;
    } else if (iequal(arg, "epsilon2Large")) {
      need(1);
      s.epsilon2Large = std::atof(tok[1].c_str());
    } else if (iequal(arg, "sampleN")) {
      need(1);
      s.sampleN = std::atoi(tok[1].c_str());
    } else if (iequal(arg, "nPTiter")) {
      need(1);
      s.nPTiter = std::atoi(tok[1].c_str());
    } else if (iequal(arg, "targetError")) {
      need(1);
      s.targetError = std::atof(tok[1].c_str());
    } else if (iequal(arg, "Treversal")) {  // SHCI/input.cpp:253-258
      need(1);
      s.trev = std::atoi(tok[1].c_str());
      if (!(s.trev == 0 || s.trev == 1 || s.trev == -1))
        throw Error(kErrInvalid, "Treversal should be either 0, 1, or -1.");
    } else if (iequal(arg, "io")) {
      s.io = true;
    } else if (iequal(arg, "noio")) {
      s.io = false;
    } else if (iequal(arg, "restart")) {
      s.restart = 1;
    } else if (iequal(arg, "fullrestart")) {
      s.restart = 2;
    } else if (iequal(arg, "prefix")) {
      need(1);
      s.prefix = tok[1];
    } else if (iequal(arg, "writebestdeterminants")) {
      need(1);
      s.writeBest = std::atoi(tok[1].c_str());
    } else if (iequal(arg, "seed")) {
      need(1);
      s.seed = std::atoll(tok[1].c_str());
    } else if (iequal(arg, "blockdavidson")) {
      s.block = true;
    } else if (iequal(arg, "precond")) {
      need(1);
      if (iequal(tok[1], "plain") || iequal(tok[1], "diagonal"))
        s.precond = 0;
      else if (iequal(tok[1], "pt2"))
        s.precond = 1;
      else if (iequal(tok[1], "mlp"))
        s.precond = 2;
      else
        throw Error(kErrInvalid, "precond must be plain, pt2 or mlp");
    } else if (iequal(arg, "davidsonBasis")) {
      need(2);
      s.basis_max = std::atoi(tok[1].c_str());
      s.basis_keep = std::atoi(tok[2].c_str());
      if (s.basis_max < 3 || s.basis_max > 16 || s.basis_keep < 1 || s.basis_keep >= s.basis_max)
        throw Error(kErrInvalid, "davidsonBasis needs max in 3..16 and keep in 1..max-1");
    } else {
      bool ok = false;
      for (const char* k : kIgnored)
        if (iequal(arg, k)) ok = true;
      if (!ok) throw Error(kErrInvalid, "cannot read option " + arg);
    }
  }
  if (sweep_iter.empty()) throw Error(kErrInvalid, "schedule block missing");
  if (maxiter < sweep_iter.back()) throw Error(kErrInvalid, "maxiter should be greater than last entry of sweep_iter");
  if (nocc == -1) throw Error(kErrInvalid, "nocc keyword has to be included.");
  if (s.direct) s.davidsonTolLoose = 3.e-2;
  s.epsilon1.clear();
  for (size_t i = 1; i < sweep_iter.size(); i++)
    for (int j = sweep_iter[i - 1]; j < sweep_iter[i]; j++) s.epsilon1.push_back(sweep_eps[i - 1]);
  for (int j = sweep_iter.back(); j < maxiter; j++) s.epsilon1.push_back(sweep_eps.back());
  if (s.epsilon1.empty()) throw Error(kErrInvalid, "eps1 schedule is empty (maxiter too small)");
  if (s.restrictions.size() > 4) throw Error(kErrInvalid, "at most 4 occupation restrictions are supported");
}

}  // namespace shci

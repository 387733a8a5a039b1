// SHCI variational oracle: a CPU restatement of Dice's variational path.
//
// TEST INFRASTRUCTURE ONLY. This file is the checker for the GPU library in
// dice_gb300/: only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline leg may load it. Nothing in the product links or calls it.
//
// Every function below restates one piece of the reference (sanshar/Dice,
// directory SHCI/) and cites the file:line it follows. Arithmetic order is
// kept where it decides bits: the FP32 cast and ordering of the heat-bath
// lists, the threshold comparisons of the selection, the summation order of
// the single-excitation matrix element and of the diagonal energy.
//
// Parity pins (checked by tests/test_oracle_golden.py against data copied
// from the reference's own tests/examples): examples/h8_631g (per-iteration
// determinant counts, the final determinant set, E_var), tests/SHCI/restart
// (E_var), tests/SHCI/n2_RAS (E_var with an occupation restriction).
//
// Determinants are two 64-bit words (up to 64 spatial orbitals), spin-orbital
// p at bit p%64 of word p/64, alpha = even p, beta = odd p, as in
// SHCI/Determinants.h:247-602.

#include <algorithm>
#include <atomic>
#include <random>
#include <cassert>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <numeric>
#include <sstream>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace orc {

static const int W = 2;
struct Det {
  uint64_t w[W];
};

static inline bool det_less(const Det& a, const Det& b) {
  // Determinant::operator< (SHCI/Determinants.h:490-498): words compared as
  // signed long from the top word down.
  for (int i = W - 1; i >= 0; --i) {
    int64_t x = (int64_t)a.w[i], y = (int64_t)b.w[i];
    if (x < y) return true;
    if (x > y) return false;
  }
  return false;
}
static inline bool det_eq(const Det& a, const Det& b) {
  for (int i = 0; i < W; ++i)
    if (a.w[i] != b.w[i]) return false;
  return true;
}
static inline bool getocc(const Det& d, int p) { return (d.w[p >> 6] >> (p & 63)) & 1ull; }
static inline void setocc(Det& d, int p, bool v) {
  if (v)
    d.w[p >> 6] |= (1ull << (p & 63));
  else
    d.w[p >> 6] &= ~(1ull << (p & 63));
}
static inline int popc(uint64_t x) { return __builtin_popcountll(x); }

// ---------------------------------------------------------------------------
// Integrals (SHCI/integral.h:47-102, SHCI/integral.cpp:43-225)
// ---------------------------------------------------------------------------
struct Ints {
  int norb = 0;   // spatial orbitals
  int nelec = 0;
  double coreE = 0.0;
  std::vector<double> I1;  // (2n)x(2n) spin-orbital one-electron matrix
  std::vector<double> I2;  // 8-fold packed (ij|kl), spatial
  std::vector<double> Direct, Exchange;  // n x n
  double maxEntry = 100.0;
  std::vector<int> irrep;

  // twoInt::operator() (SHCI/integral.h:86-101), non-ksym branch
  inline double i2(int i, int j, int k, int l) const {
    if (!((i % 2 == j % 2) && (k % 2 == l % 2))) return 0.0;
    int I = i / 2, J = j / 2, K = k / 2, L = l / 2;
    int IJ = std::max(I, J) * (std::max(I, J) + 1) / 2 + std::min(I, J);
    int KL = std::max(K, L) * (std::max(K, L) + 1) / 2 + std::min(K, L);
    size_t A = std::max(IJ, KL), B = std::min(IJ, KL);
    return I2[A * (A + 1) / 2 + B];
  }
  inline double& i2ref_spatial(int I, int J, int K, int L) {
    int IJ = std::max(I, J) * (std::max(I, J) + 1) / 2 + std::min(I, J);
    int KL = std::max(K, L) * (std::max(K, L) + 1) / 2 + std::min(K, L);
    size_t A = std::max(IJ, KL), B = std::min(IJ, KL);
    return I2[A * (A + 1) / 2 + B];
  }
  inline double i1(int i, int j) const { return I1[(size_t)i * (2 * norb) + j]; }
  inline double direct(int i, int j) const { return Direct[(size_t)i * norb + j]; }
  inline double exchange(int i, int j) const { return Exchange[(size_t)i * norb + j]; }
};

// boost::trim + boost::split(tok, line, is_any_of(delims), token_compress_on)
static void split_compress(const std::string& in, const char* delims, std::vector<std::string>& tok) {
  size_t b = 0, e = in.size();
  while (b < e && isspace((unsigned char)in[b])) ++b;
  while (e > b && isspace((unsigned char)in[e - 1])) --e;
  std::string s = in.substr(b, e - b);
  tok.clear();
  std::string cur;
  bool last_delim = false;
  for (size_t i = 0; i < s.size(); ++i) {
    if (strchr(delims, s[i])) {
      if (!last_delim) {
        tok.push_back(cur);
        cur.clear();
      }
      last_delim = true;
    } else {
      cur.push_back(s[i]);
      last_delim = false;
    }
  }
  tok.push_back(cur);
}
static bool iequals(const std::string& a, const std::string& b) {
  if (a.size() != b.size()) return false;
  for (size_t i = 0; i < a.size(); ++i)
    if (tolower((unsigned char)a[i]) != tolower((unsigned char)b[i])) return false;
  return true;
}

// readIntegrals (SHCI/integral.cpp:43-225), serial branch.
static int read_fcidump(const char* path, Ints& I, std::string& err) {
  std::ifstream dump(path);
  if (!dump.good()) {
    err = std::string("Integral file ") + path + " does not exist!";
    return 1;
  }
  int norbs = -1, nelec = -1;
  std::vector<std::string> tok;
  std::string msg;
  while (!dump.eof()) {
    std::getline(dump, msg);
    split_compress(msg, ", \t=", tok);
    if (tok.size() == 1 && (iequals(tok[0], "&END") || iequals(tok[0], "/"))) break;
    if (iequals(tok[0].substr(0, 4), "&FCI")) {
      if (tok.size() > 2 && iequals(tok[1].substr(0, 4), "NORB")) norbs = atoi(tok[2].c_str());
      if (tok.size() > 4 && iequals(tok[3].substr(0, 5), "NELEC")) nelec = atoi(tok[4].c_str());
    } else if (iequals(tok[0].substr(0, 4), "ISYM")) {
      continue;
    } else if (iequals(tok[0].substr(0, 4), "KSYM")) {
      err = "KSYM integrals are not supported";
      return 2;
    } else if (iequals(tok[0].substr(0, 6), "ORBSYM")) {
      for (size_t i = 1; i < tok.size(); i++) I.irrep.push_back(atoi(tok[i].c_str()));
    } else {
      for (size_t i = 0; i < tok.size(); i++) I.irrep.push_back(atoi(tok[i].c_str()));
    }
  }
  if (norbs == -1 || nelec == -1) {
    err = "could not read the norbs or nelec";
    return 3;
  }
  if (norbs > 64) {
    err = "more than 64 spatial orbitals";
    return 4;
  }
  I.irrep.resize(norbs);
  I.norb = norbs;
  I.nelec = nelec;
  size_t npair = (size_t)norbs * (norbs + 1) / 2;
  I.I2.assign(npair * (npair + 1) / 2, 0.0);
  I.I1.assign((size_t)(2 * norbs) * (2 * norbs), 0.0);
  I.coreE = 0.0;
  const int n2 = 2 * norbs;
  while (!dump.eof()) {
    std::getline(dump, msg);
    split_compress(msg, ", \t", tok);
    if (tok.size() != 5) continue;
    double integral = atof(tok[0].c_str());
    int a = atoi(tok[1].c_str()), b = atoi(tok[2].c_str()), c = atoi(tok[3].c_str()),
        d = atoi(tok[4].c_str());
    if (a == b && b == c && c == d && d == 0) {
      I.coreE = integral;
    } else if (b == c && c == d && d == 0) {
      continue;
    } else if (c == d && d == 0) {
      if (a < 1 || b < 1 || a > norbs || b > norbs) continue;
      I.I1[(size_t)(2 * (a - 1)) * n2 + 2 * (b - 1)] = integral;
      I.I1[(size_t)(2 * (a - 1) + 1) * n2 + 2 * (b - 1) + 1] = integral;
      I.I1[(size_t)(2 * (b - 1)) * n2 + 2 * (a - 1)] = integral;
      I.I1[(size_t)(2 * (b - 1) + 1) * n2 + 2 * (a - 1) + 1] = integral;
    } else {
      if (a < 1 || b < 1 || c < 1 || d < 1 || a > norbs || b > norbs || c > norbs || d > norbs) continue;
      I.i2ref_spatial(a - 1, b - 1, c - 1, d - 1) = integral;
    }
  }
  // maxEntry: element of largest magnitude (SHCI/integral.cpp:38, :170-171)
  double best = I.I2.empty() ? 0.0 : I.I2[0];
  for (double v : I.I2)
    if (fabs(best) < fabs(v)) best = v;
  I.maxEntry = best;
  I.Direct.assign((size_t)norbs * norbs, 0.0);
  I.Exchange.assign((size_t)norbs * norbs, 0.0);
  for (int i = 0; i < norbs; i++)
    for (int j = 0; j < norbs; j++) {
      I.Direct[(size_t)i * norbs + j] = I.i2(2 * i, 2 * i, 2 * j, 2 * j);
      I.Exchange[(size_t)i * norbs + j] = I.i2(2 * i, 2 * j, 2 * j, 2 * i);
    }
  return 0;
}

// ---------------------------------------------------------------------------
// Heat-bath tables (SHCI/integral.h:125-153, SHCI/integral.cpp:228-389)
// ---------------------------------------------------------------------------
struct HeatBath {
  std::vector<float> sameVal, oppVal;
  std::vector<int16_t> samePairs, oppPairs;  // (a,b) per entry
  std::vector<uint64_t> sameStart, oppStart;  // n(n+1)/2 + 1
  std::vector<double> Singles;               // (2n)x(2n)
};

// One pair list: entries inserted in (a,b) order into a multimap keyed by
// |float| (compAbs), read back by reverse iteration. That is: |v| descending,
// equal |v| in reverse insertion order.
struct HBEntry {
  float v;
  int16_t a, b;
  int seq;
};
static void hb_emit(std::vector<HBEntry>& e, std::vector<float>& vals, std::vector<int16_t>& pairs) {
  std::sort(e.begin(), e.end(), [](const HBEntry& x, const HBEntry& y) {
    float ax = fabsf(x.v), ay = fabsf(y.v);
    if (ax != ay) return ax > ay;
    return x.seq > y.seq;
  });
  for (auto& x : e) {
    vals.push_back(x.v);
    pairs.push_back(x.a);
    pairs.push_back(x.b);
  }
}

static void build_heatbath(const Ints& I, HeatBath& hb) {
  const int n = I.norb;
  const double eps = 1.e-10;  // twoIntHeatBath(1.e-10) at SHCI/SHCI.cpp:247
  hb.sameStart.assign(1, 0);
  hb.oppStart.assign(1, 0);
  std::vector<HBEntry> same, opp;
  for (int i = 0; i < n; i++)
    for (int j = 0; j <= i; j++) {
      same.clear();
      opp.clear();
      int seqs = 0, seqo = 0;
      for (int a = 0; a < n; a++)
        for (int b = 0; b < n; b++) {
          double v = I.i2(2 * i, 2 * a, 2 * j, 2 * b);
          if (fabs(v) > eps) opp.push_back({(float)v, (int16_t)a, (int16_t)b, seqo++});
          if (a >= b) {
            double s = I.i2(2 * i, 2 * a, 2 * j, 2 * b) - I.i2(2 * i, 2 * b, 2 * j, 2 * a);
            if (fabs(s) > eps) same.push_back({(float)s, (int16_t)a, (int16_t)b, seqs++});
          }
        }
      hb_emit(same, hb.sameVal, hb.samePairs);
      hb_emit(opp, hb.oppVal, hb.oppPairs);
      hb.sameStart.push_back(hb.sameVal.size());
      hb.oppStart.push_back(hb.oppVal.size());
    }
  const int n2 = 2 * n;
  hb.Singles.assign((size_t)n2 * n2, 0.0);
  for (int i = 0; i < n2; i++)
    for (int a = 0; a < n2; a++) {
      double s = fabs(I.i1(i, a));
      for (int j = 0; j < n2; j++) {
        double t = I.i2(i, a, j, j) - I.i2(i, j, j, a);
        if (fabs(s) < fabs(t)) s = fabs(t);
      }
      hb.Singles[(size_t)i * n2 + a] = s;
    }
}

// ---------------------------------------------------------------------------
// Slater-Condon rules (SHCI/Determinants.cpp:252-300, :406-505, :564-631)
// ---------------------------------------------------------------------------
static int closed_list(const Det& d, int nspin, int* closed) {
  int c = 0;
  for (int p = 0; p < nspin; ++p)
    if (getocc(d, p)) closed[c++] = p;
  return c;
}

// Determinant::Energy, coreE excluded (SHCI/Determinants.cpp:252-300)
static double det_energy(const Ints& I, const Det& d) {
  int closed[128];
  int nc = closed_list(d, 2 * I.norb, closed);
  double energy = 0.0;
  for (int i = 0; i < nc; i++) {
    int P = closed[i];
    energy += I.i1(P, P);
    for (int j = i + 1; j < nc; j++) {
      int Q = closed[j];
      energy += I.direct(P / 2, Q / 2);
      if ((P % 2) == (Q % 2)) energy -= I.exchange(P / 2, Q / 2);
    }
  }
  return energy;
}

// Determinant::parity(start,end) (SHCI/Determinants.h:283-301): sign of the
// number of occupied spin orbitals strictly between start and end.
static double parity_between(const Det& d, int lo, int hi) {
  int cnt = 0;
  for (int p = lo + 1; p < hi; ++p) cnt += getocc(d, p);
  return (cnt & 1) ? -1.0 : 1.0;
}

// Hij_1Excite(a, i, ..., closed, nclosed) (SHCI/Determinants.cpp:437-469):
// a created, i destroyed; sum runs over the ket's occupied list in order.
static double hij_1excite(const Ints& I, int a, int i, const int* closed, int nclosed) {
  double sgn = 1.0;
  double energy = I.i1(a, i);
  int lo = std::min(i, a), hi = std::max(i, a);
  for (int j = 0; j < nclosed; j++) {
    if (closed[j] > lo && closed[j] < hi) sgn *= -1.;
    energy += (I.i2(a, i, closed[j], closed[j]) - I.i2(a, closed[j], closed[j], i));
  }
  return energy * sgn;
}

// Determinant::Hij_2Excite(i, j, a, b) (SHCI/Determinants.cpp:406-434)
static double hij_2excite(const Ints& I, const Det& ket, int i, int j, int a, int b) {
  double sgn = 1.0;
  int II = std::min(i, j), JJ = std::max(i, j), A = std::min(a, b), B = std::max(a, b);
  sgn *= parity_between(ket, std::min(II, A), std::max(II, A));
  sgn *= parity_between(ket, std::min(JJ, B), std::max(JJ, B));
  if (A > JJ || B < II) sgn *= -1.;
  return sgn * (I.i2(A, II, B, JJ) - I.i2(A, JJ, B, II));
}

// Hij(bra, ket) (SHCI/Determinants.cpp:564-631)
static double hij(const Ints& I, const Det& bra, const Det& ket) {
  int cre[4], des[4], ncre = 0, ndes = 0;
  for (int w = 0; w < W; ++w) {
    uint64_t u = bra.w[w] ^ ket.w[w];
    uint64_t b = u & bra.w[w], k = u & ket.w[w];
    while (b) {
      int pos = __builtin_ctzll(b);
      if (ncre < 4) cre[ncre] = pos + 64 * w;
      ncre++;
      b &= b - 1;
    }
    while (k) {
      int pos = __builtin_ctzll(k);
      if (ndes < 4) des[ndes] = pos + 64 * w;
      ndes++;
      k &= k - 1;
    }
  }
  if (ncre == 1) {
    int closed[128];
    int nc = closed_list(ket, 2 * I.norb, closed);
    // ket.Hij_1Excite(cre, des) sums over the ket's occupied orbitals
    // (SHCI/Determinants.cpp:472-505); same arithmetic as the free function.
    return hij_1excite(I, cre[0], des[0], closed, nc);
  } else if (ncre == 2) {
    return hij_2excite(I, ket, des[0], des[1], cre[0], cre[1]);
  }
  return 0.0;
}

static inline int excitation_distance(const Det& a, const Det& b) {
  int n = 0;
  for (int w = 0; w < W; ++w) n += popc(a.w[w] ^ b.w[w]);
  return n / 2;
}

// ---------------------------------------------------------------------------
// Occupation restrictions (SHCI/OccRestrictions.cpp)
// ---------------------------------------------------------------------------
struct Restriction {
  int minElec, maxElec;
  std::vector<int> orbs;  // spin orbitals
  int currentElec = 0;
};
static void restrictions_init(std::vector<Restriction>& rs, const int* closed, int nc) {
  for (auto& r : rs) {
    r.currentElec = 0;
    for (int i = 0; i < nc; i++)
      for (int o : r.orbs)
        if (o == closed[i]) r.currentElec++;
  }
}
static bool restr_one(const std::vector<Restriction>& rs, int i, int a) {
  for (auto& r : rs) {
    int e = r.currentElec;
    for (int o : r.orbs) {
      if (o == i) e--;
      if (o == a) e++;
    }
    if (e < r.minElec || e > r.maxElec) return false;
  }
  return true;
}
static bool restr_two(const std::vector<Restriction>& rs, int i, int j, int a, int b) {
  for (auto& r : rs) {
    int e = r.currentElec;
    for (int o : r.orbs) {
      if (o == i || o == j) e--;
      if (o == a || o == b) e++;
    }
    if (e < r.minElec || e > r.maxElec) return false;
  }
  return true;
}

// Worker threads of the oracle's timed reference run (orc_set_threads); 1 for
// the serial restatement every parity test uses. Threads stand in for the
// MPI ranks of one node: selection deals parents, the build deals rows and
// sigma is the reference's rank-parallel Hmult2 (sigma_mt below).
static int g_threads = 1;

// Runs f(b) for b in [0, nblocks) on g_threads workers (blocks handed out in
// order from a shared counter); serial when g_threads == 1.
template <class F>
static void parallel_blocks(size_t nblocks, F&& f) {
  const int T = std::max(1, std::min<int>(g_threads, (int)std::max<size_t>(1, nblocks)));
  if (T == 1) {
    for (size_t b = 0; b < nblocks; ++b) f(b);
    return;
  }
  std::atomic<size_t> next{0};
  std::vector<std::thread> pool;
  for (int w = 0; w < T; ++w)
    pool.emplace_back([&] {
      for (size_t b; (b = next.fetch_add(1)) < nblocks;) f(b);
    });
  for (auto& th : pool) th.join();
}

struct SelParams {
  int ncore = 0;
  int nact = 1000000;
  std::vector<Restriction> restrictions;
};

// SHCIgetdeterminants::getDeterminantsVariationalApprox
// (SHCI/SHCIgetdeterminants.cpp:586-739)
static void select_from_parent(const Ints& I, const HeatBath& hb, const Det& d, double epsilon,
                               SelParams& sp, const Det* sorted, size_t nsorted,
                               std::vector<Det>& out) {
  const int nspin = 2 * I.norb;
  int closed[128], open[128];
  int nclosed = 0, nopen = 0;
  for (int p = 0; p < nspin; ++p) {
    if (getocc(d, p))
      closed[nclosed++] = p;
    else
      open[nopen++] = p;
  }
  restrictions_init(sp.restrictions, closed, nclosed);
  auto present = [&](const Det& x) {
    return std::binary_search(sorted, sorted + nsorted, x, det_less);
  };
  const int n2 = nspin;
  for (int ia = 0; ia < nopen * nclosed; ia++) {
    int i = ia / nopen, a = ia % nopen;
    if (closed[i] / 2 < sp.ncore || open[a] / 2 >= sp.ncore + sp.nact) continue;
    if (!restr_one(sp.restrictions, closed[i], open[a])) continue;
    double integral = hb.Singles[(size_t)open[a] * n2 + closed[i]];
    if (fabs(integral) > epsilon)
      if (closed[i] % 2 == open[a] % 2)
        integral = hij_1excite(I, open[a], closed[i], closed, nclosed);
    if (fabs(integral) > epsilon) {
      Det di = d;
      setocc(di, open[a], true);
      setocc(di, closed[i], false);
      if (!present(di)) out.push_back(di);
    }
  }
  if (fabs(I.maxEntry) < epsilon) return;
  for (int ij = 0; ij < nclosed * nclosed; ij++) {
    int i = ij / nclosed, j = ij % nclosed;
    if (i <= j) continue;
    int Ii = closed[i] / 2, Jj = closed[j] / 2;
    int X = std::max(Ii, Jj), Y = std::min(Ii, Jj);
    if (closed[i] / 2 < sp.ncore || closed[j] / 2 < sp.ncore) continue;
    int pairIndex = X * (X + 1) / 2 + Y;
    bool same = closed[i] % 2 == closed[j] % 2;
    size_t start = same ? hb.sameStart[pairIndex] : hb.oppStart[pairIndex];
    size_t end = same ? hb.sameStart[pairIndex + 1] : hb.oppStart[pairIndex + 1];
    const float* integrals = same ? hb.sameVal.data() : hb.oppVal.data();
    const int16_t* orbIndices = same ? hb.samePairs.data() : hb.oppPairs.data();
    for (size_t index = start; index < end; index++) {
      if (fabsf(integrals[index]) < epsilon) break;
      int a = 2 * orbIndices[2 * index] + closed[i] % 2;
      int b = 2 * orbIndices[2 * index + 1] + closed[j] % 2;
      if (a / 2 >= sp.ncore + sp.nact || b / 2 >= sp.ncore + sp.nact) continue;
      if (!restr_two(sp.restrictions, closed[i], closed[j], a, b)) continue;
      if (!(getocc(d, a) || getocc(d, b))) {
        Det di = d;
        setocc(di, a, true);
        setocc(di, b, true);
        setocc(di, closed[i], false);
        setocc(di, closed[j], false);
        if (!present(di)) out.push_back(di);
      }
    }
  }
}

// Selection over all parents + sort/unique (SHCI/SHCIbasics.cpp:954-994)
static void select_all(const Ints& I, const HeatBath& hb, const Det* dets, size_t n, const double* cmax,
                       double eps1, SelParams& sp, const Det* sorted, size_t nsorted,
                       std::vector<Det>& newdets) {
  newdets.clear();
  if (g_threads <= 1) {
    for (size_t i = 0; i < n; i++)
      select_from_parent(I, hb, dets[i], eps1 / fabs(cmax[i]), sp, sorted, nsorted, newdets);
  } else {  // parents dealt in blocks; the candidates are sorted and uniqued below either way
    const size_t kPar = 256, nblk = (n + kPar - 1) / kPar;
    std::vector<std::vector<Det>> part(nblk);
    parallel_blocks(nblk, [&](size_t b) {
      SelParams spl = sp;  // restrictions_init rewrites it per parent
      for (size_t i = b * kPar; i < std::min(n, (b + 1) * kPar); i++)
        select_from_parent(I, hb, dets[i], eps1 / fabs(cmax[i]), spl, sorted, nsorted, part[b]);
      std::sort(part[b].begin(), part[b].end(), det_less);
      part[b].erase(std::unique(part[b].begin(), part[b].end(), det_eq), part[b].end());
    });
    for (auto& v : part) {
      newdets.insert(newdets.end(), v.begin(), v.end());
      std::vector<Det>().swap(v);
    }
  }
  std::sort(newdets.begin(), newdets.end(), det_less);
  newdets.erase(std::unique(newdets.begin(), newdets.end(), det_eq), newdets.end());
}

// ---------------------------------------------------------------------------
// Deterministic second-order (Epstein-Nesbet) perturbation theory
// ---------------------------------------------------------------------------
// EnergyAfterExcitation, single i -> A (SHCI/Determinants.cpp:124-172):
// the excited determinant's energy from the parent's, i the index into closed.
static double energy_after_single(const Ints& I, const int* closed, int nclosed, int i, int A, double Energyd) {
  double E = Energyd;
  E += -I.i1(closed[i], closed[i]) + I.i1(A, A);
  for (int k = 0; k < nclosed; k++) {
    if (k == i) continue;
    E = E - I.direct(closed[k] / 2, closed[i] / 2) + I.direct(closed[k] / 2, A / 2);
    if ((closed[k] % 2) == (closed[i] % 2))
      E = E + I.exchange(closed[k] / 2, closed[i] / 2) - I.exchange(closed[k] / 2, A / 2);
  }
  return E;
}

// EnergyAfterExcitation, double i -> A, j -> B (SHCI/Determinants.cpp:178-249).
static double energy_after_double(const Ints& I, const int* closed, int nclosed, int i, int A, int j, int B,
                                  double Energyd) {
  double E = Energyd - I.i1(closed[i], closed[i]) + I.i1(A, A) - I.i1(closed[j], closed[j]) + I.i1(B, B);
  for (int k = 0; k < nclosed; k++) {
    if (k == i) continue;
    E = E - I.direct(closed[k] / 2, closed[i] / 2) + I.direct(closed[k] / 2, A / 2);
    if ((closed[k] % 2) == (closed[i] % 2))
      E = E + I.exchange(closed[k] / 2, closed[i] / 2) - I.exchange(closed[k] / 2, A / 2);
  }
  for (int k = 0; k < nclosed; k++) {
    if (k == i || k == j) continue;
    E = E - I.direct(closed[k] / 2, closed[j] / 2) + I.direct(closed[k] / 2, B / 2);
    if ((closed[k] % 2) == (closed[j] % 2))
      E = E + I.exchange(closed[k] / 2, closed[j] / 2) - I.exchange(closed[k] / 2, B / 2);
  }
  E = E - I.direct(A / 2, closed[j] / 2) + I.direct(A / 2, B / 2);
  if ((closed[i] % 2) == (closed[j] % 2)) E = E + I.exchange(A / 2, closed[j] / 2) - I.exchange(A / 2, B / 2);
  return E;
}

// Determinant::parity(a, b, i, j, sgn) evaluated on the excited determinant
// di (SHCI/Determinants.cpp:332-357, called at
// SHCI/SHCIgetdeterminants.cpp:155-157): the a<->i transposition counted on
// di, then the b<->j one on di with a emptied and i refilled.
static double pt_double_sign(Det di, int a, int b, int i, int j) {
  double sgn = parity_between(di, std::min(a, i), std::max(a, i));
  setocc(di, a, false);
  setocc(di, i, true);
  sgn *= parity_between(di, std::min(b, j), std::max(b, j));
  return sgn;
}

struct PtCand {
  Det d;
  double num;
  double E;
};

// SHCIgetdeterminants::getDeterminantsDeterministicPT
// (SHCI/SHCIgetdeterminants.cpp:40-171): every single above epsilon by its
// exact matrix element, every double whose heat-bath |float| is >= epsilon;
// numerator H_ai c_i (the double's from the FP32 list value), energy by
// EnergyAfterExcitation. No ncore/nact filter: only the PT restrictions.
static void pt_from_parent(const Ints& I, const HeatBath& hb, const Det& d, double epsilon, double ci1,
                           std::vector<Restriction>& rs, std::vector<PtCand>& out) {
  const int nspin = 2 * I.norb;
  int closed[128], open[128];
  int nclosed = 0, nopen = 0;
  for (int p = 0; p < nspin; ++p) {
    if (getocc(d, p))
      closed[nclosed++] = p;
    else
      open[nopen++] = p;
  }
  const double Energyd = det_energy(I, d) + I.coreE;
  restrictions_init(rs, closed, nclosed);
  for (int ia = 0; ia < nopen * nclosed; ia++) {
    int i = ia / nopen, a = ia % nopen;
    if (!restr_one(rs, closed[i], open[a])) continue;
    double integral = hij_1excite(I, open[a], closed[i], closed, nclosed);
    if (closed[i] % 2 != open[a] % 2) {
      // spin flip: I1 has no alpha-beta block, so the element is zero
      double sgn = parity_between(d, std::min(open[a], closed[i]), std::max(open[a], closed[i]));
      integral = I.i1(open[a], closed[i]) * sgn;
    }
    if (fabs(integral) > epsilon) {
      PtCand c;
      c.d = d;
      setocc(c.d, open[a], true);
      setocc(c.d, closed[i], false);
      c.num = integral * ci1;
      c.E = energy_after_single(I, closed, nclosed, i, open[a], Energyd);
      out.push_back(c);
    }
  }
  if (fabs(I.maxEntry) < epsilon) return;
  for (int ij = 0; ij < nclosed * nclosed; ij++) {
    int i = ij / nclosed, j = ij % nclosed;
    if (i <= j) continue;
    int Ii = closed[i] / 2, Jj = closed[j] / 2;
    int X = std::max(Ii, Jj), Y = std::min(Ii, Jj);
    int pairIndex = X * (X + 1) / 2 + Y;
    bool same = closed[i] % 2 == closed[j] % 2;
    size_t start = same ? hb.sameStart[pairIndex] : hb.oppStart[pairIndex];
    size_t end = same ? hb.sameStart[pairIndex + 1] : hb.oppStart[pairIndex + 1];
    const float* integrals = same ? hb.sameVal.data() : hb.oppVal.data();
    const int16_t* orbIndices = same ? hb.samePairs.data() : hb.oppPairs.data();
    for (size_t index = start; index < end; index++) {
      if (fabsf(integrals[index]) < epsilon) break;
      int a = 2 * orbIndices[2 * index] + closed[i] % 2;
      int b = 2 * orbIndices[2 * index + 1] + closed[j] % 2;
      if (!restr_two(rs, closed[i], closed[j], a, b)) continue;
      if (!(getocc(d, a) || getocc(d, b))) {
        PtCand c;
        c.d = d;
        setocc(c.d, a, true);
        setocc(c.d, b, true);
        setocc(c.d, closed[i], false);
        setocc(c.d, closed[j], false);
        double sgn = pt_double_sign(c.d, a, b, closed[i], closed[j]);
        c.num = integrals[index] * sgn * ci1;
        c.E = energy_after_double(I, closed, nclosed, i, a, j, b, Energyd);
        out.push_back(c);
      }
    }
  }
}

struct PtStats {
  int64_t candidates = 0, unique = 0;
  int64_t outside = 0;  // candidates not in the variational space, before merging
  double psi1_norm = 0.0;
};

// SHCIbasics::DoPerturbativeDeterministic (SHCI/SHCIbasics.cpp:453-728),
// serial, without the RDM/response branch: candidates of every parent with
// epsilon = |eps2 / c_i|, stable sort by determinant, duplicates merged by
// summing numerators in generation order (StitchDEH::MergeSortAndRemoveDuplicates,
// SHCI/SHCISortMpiUtils.cpp:541-640), determinants of the variational space
// removed (StitchDEH::RemoveDetsPresentIn, :750-800), then
// E2 = sum |N_a|^2 / (E0 - E_a). E0 and the energies include coreE.
// Parents [p0, p1) only when p1 > p0 (a bounded sample for timing); the
// whole space is still removed from the candidates.
static double pt_deterministic(const Ints& I, const HeatBath& hb, const Det* dets, size_t n, const double* ci,
                               double E0, double eps2, std::vector<Restriction> rs, PtStats& st, size_t p0 = 0,
                               size_t p1 = 0) {
  std::vector<PtCand> all;
  if (p1 <= p0) {
    p0 = 0;
    p1 = n;
  }
  for (size_t i = p0; i < p1 && i < n; i++) pt_from_parent(I, hb, dets[i], fabs(eps2 / ci[i]), ci[i], rs, all);
  st.candidates = (int64_t)all.size();
  st.outside = 0;
  std::stable_sort(all.begin(), all.end(), [](const PtCand& x, const PtCand& y) { return det_less(x.d, y.d); });
  std::vector<Det> sorted(dets, dets + n);
  std::sort(sorted.begin(), sorted.end(), det_less);
  double e2 = 0.0, psi = 0.0;
  int64_t uniq = 0;
  size_t k = 0, v = 0;
  while (k < all.size()) {
    size_t e = k + 1;
    double num = all[k].num;
    while (e < all.size() && det_eq(all[e].d, all[k].d)) num += all[e++].num;
    while (v < sorted.size() && det_less(sorted[v], all[k].d)) ++v;
    bool present = v < sorted.size() && det_eq(sorted[v], all[k].d);
    if (!present) {
      st.outside += (int64_t)(e - k);
      const double de = E0 - all[k].E;
      psi += pow(fabs(num / de), 2);
      e2 += pow(fabs(num), 2) / de;
      ++uniq;
    }
    k = e;
  }
  st.unique = uniq;
  st.psi1_norm = psi;
  return e2;
}

// ---------------------------------------------------------------------------
// Sparse Hamiltonian: lower triangle with diagonal first, as SparseHam holds it
// (SHCI/SHCImakeHamiltonian.cpp:486-715). Connections are every J < I at
// excitation distance 1 or 2; values Hij(Dets[J], Dets[I]).
// The reference finds them through alpha/beta string helper lists
// (:184-408); the oracle finds the same set by grouping on strings too.
// ---------------------------------------------------------------------------
struct SparseHam {
  std::vector<int64_t> rowptr;  // N+1
  std::vector<int32_t> col;
  std::vector<double> val;
};

static inline uint64_t spin_string(const Det& d, int s) {
  // getAlpha/getBeta (SHCI/Determinants.h:471-487): orbital k of spin s is
  // spin-orbital 2k+s.
  uint64_t out = 0;
  for (int w = 0; w < W; ++w) {
    uint64_t x = d.w[w] >> s;
    for (int k = 0; k < 32; ++k)
      if ((x >> (2 * k)) & 1ull) out |= 1ull << (32 * w + k);
  }
  return out;
}

// Rows [n_old, N) of the lower triangle (the rows of the first n_old
// determinants are kept: selection only appends, and row I holds J <= I), as
// SparseHam::makeFromHelper builds the rows from StartIndex on
// (SHCI/SHCImakeHamiltonian.cpp:486-715). n_old = 0 builds every row.
// stride > 1 keeps only the rows I with I % stride == 0 (the others are left
// empty): a bounded sample of the space's rows for timing the sigma.
static void build_ham(const Ints& I, const Det* dets, size_t N, SparseHam& H, size_t n_old = 0,
                      size_t stride = 1) {
  std::unordered_map<uint64_t, int> amap, bmap;
  std::vector<uint64_t> astr, bstr;
  std::vector<int> aidx(N), bidx(N);
  for (size_t k = 0; k < N; ++k) {
    uint64_t a = spin_string(dets[k], 0), b = spin_string(dets[k], 1);
    auto ia = amap.emplace(a, (int)astr.size());
    if (ia.second) astr.push_back(a);
    auto ib = bmap.emplace(b, (int)bstr.size());
    if (ib.second) bstr.push_back(b);
    aidx[k] = ia.first->second;
    bidx[k] = ib.first->second;
  }
  std::vector<std::vector<int>> byA(astr.size()), byB(bstr.size());
  for (size_t k = 0; k < N; ++k) {
    byA[aidx[k]].push_back((int)k);
    byB[bidx[k]].push_back((int)k);
  }
  // single-excitation neighbours among the present alpha strings
  const int n = I.norb;
  std::vector<std::vector<int>> singA(astr.size());
  parallel_blocks((astr.size() + 1023) / 1024, [&](size_t blk) {
    for (size_t s = blk * 1024; s < std::min(astr.size(), (blk + 1) * 1024); ++s) {
      uint64_t x = astr[s];
      for (int i = 0; i < n; ++i) {
        if (!((x >> i) & 1)) continue;
        for (int a = 0; a < n; ++a) {
          if ((x >> a) & 1) continue;
          uint64_t y = (x & ~(1ull << i)) | (1ull << a);
          auto it = amap.find(y);
          if (it != amap.end()) singA[s].push_back(it->second);
        }
      }
    }
  });
  if (n_old > N || H.rowptr.size() != n_old + 1) n_old = 0;
  H.rowptr.resize(N + 1);
  H.rowptr[0] = 0;
  H.col.resize((size_t)H.rowptr[n_old]);
  H.val.resize((size_t)H.rowptr[n_old]);
  // rows in blocks: each block's entries are collected privately, then the
  // blocks are appended in row order
  const size_t kRows = 2048;
  const size_t nblk = (N - n_old + kRows - 1) / kRows;
  struct Block {
    std::vector<int64_t> len;
    std::vector<int32_t> col;
    std::vector<double> val;
  };
  std::vector<Block> blocks(nblk);
  parallel_blocks(nblk, [&](size_t blk) {
    Block& B_ = blocks[blk];
    std::vector<int> row;
    const size_t r0 = n_old + blk * kRows, r1 = std::min(N, r0 + kRows);
    for (size_t I_ = r0; I_ < r1; ++I_) {
      if (stride > 1 && I_ % stride != 0) {
        B_.len.push_back(0);
        continue;
      }
      row.clear();
      const uint64_t A = astr[aidx[I_]], B = bstr[bidx[I_]];
      // same alpha string: beta single or double
      for (int J : byA[aidx[I_]]) {
        if ((size_t)J >= I_) continue;
        int d = popc(bstr[bidx[J]] ^ B);
        if (d == 2 || d == 4) row.push_back(J);
      }
      // alpha single: beta equal (single alpha) or beta single (alpha-beta double)
      for (int As : singA[aidx[I_]])
        for (int J : byA[As]) {
          if ((size_t)J >= I_) continue;
          int d = popc(bstr[bidx[J]] ^ B);
          if (d == 0 || d == 2) row.push_back(J);
        }
      // same beta string: alpha double
      for (int J : byB[bidx[I_]]) {
        if ((size_t)J >= I_) continue;
        int d = popc(astr[aidx[J]] ^ A);
        if (d == 4) row.push_back(J);
      }
      std::sort(row.begin(), row.end());
      B_.len.push_back((int64_t)row.size() + 1);
      B_.col.push_back((int32_t)I_);
      B_.val.push_back(det_energy(I, dets[I_]));
      for (int J : row) {
        B_.col.push_back(J);
        B_.val.push_back(hij(I, dets[J], dets[I_]));
      }
    }
  });
  size_t r = n_old;
  for (auto& B_ : blocks) {
    for (int64_t L : B_.len) {
      H.rowptr[r + 1] = H.rowptr[r] + L;
      ++r;
    }
    H.col.insert(H.col.end(), B_.col.begin(), B_.col.end());
    H.val.insert(H.val.end(), B_.val.begin(), B_.val.end());
    Block().col.swap(B_.col);  // release as we go
    Block().val.swap(B_.val);
  }
}

// ---------------------------------------------------------------------------
// Semistochastic PT2 (SHCIbasics::DoPerturbativeStochastic2SingleListDoubleEpsilon2AllTogether,
// SHCI/SHCIbasics.cpp:55-451)
// ---------------------------------------------------------------------------
struct PtStochCand {
  Det d;
  double num1, num2, E;
  bool present;
};

// SHCIgetdeterminants::getDeterminantsStochastic2Epsilon
// (SHCI/SHCIgetdeterminants.cpp:889-1045): the candidates of one sampled
// parent with threshold epsilon, their numerators H ci1 and
// H^2 ci1 (ci1 Nmc/(Nmc-1) - ci2), and whether |H| > epsilonLarge (the part
// the deterministic stage already holds).
static void pt_stoch_from_parent(const Ints& I, const HeatBath& hb, const Det& d, double epsilon,
                                 double epsilonLarge, double ci1, double ci2, int Nmc,
                                 std::vector<Restriction>& rs, std::vector<PtStochCand>& out) {
  const int nspin = 2 * I.norb;
  int closed[128], open[128];
  int nclosed = 0, nopen = 0;
  for (int p = 0; p < nspin; ++p) {
    if (getocc(d, p))
      closed[nclosed++] = p;
    else
      open[nopen++] = p;
  }
  const double Energyd = det_energy(I, d) + I.coreE;
  const double Nmcd = 1. * Nmc;
  restrictions_init(rs, closed, nclosed);
  for (int ia = 0; ia < nopen * nclosed; ia++) {
    int i = ia / nopen, a = ia % nopen;
    if (!restr_one(rs, closed[i], open[a])) continue;
    double integral = hij_1excite(I, open[a], closed[i], closed, nclosed);
    if (closed[i] % 2 != open[a] % 2) {
      double sgn = parity_between(d, std::min(open[a], closed[i]), std::max(open[a], closed[i]));
      integral = I.i1(open[a], closed[i]) * sgn;
    }
    if (fabs(integral) > epsilon) {
      PtStochCand c;
      c.d = d;
      setocc(c.d, open[a], true);
      setocc(c.d, closed[i], false);
      c.num1 = integral * ci1;
      c.num2 = integral * integral * ci1 * (ci1 * Nmcd / (Nmcd - 1) - ci2);
      c.E = energy_after_single(I, closed, nclosed, i, open[a], Energyd);
      c.present = fabs(integral) > epsilonLarge;
      out.push_back(c);
    }
  }
  if (fabs(I.maxEntry) < epsilon) return;
  for (int ij = 0; ij < nclosed * nclosed; ij++) {
    int i = ij / nclosed, j = ij % nclosed;
    if (i <= j) continue;
    int Ii = closed[i] / 2, Jj = closed[j] / 2;
    int X = std::max(Ii, Jj), Y = std::min(Ii, Jj);
    int pairIndex = X * (X + 1) / 2 + Y;
    bool same = closed[i] % 2 == closed[j] % 2;
    size_t start = same ? hb.sameStart[pairIndex] : hb.oppStart[pairIndex];
    size_t end = same ? hb.sameStart[pairIndex + 1] : hb.oppStart[pairIndex + 1];
    const float* integrals = same ? hb.sameVal.data() : hb.oppVal.data();
    const int16_t* orbIndices = same ? hb.samePairs.data() : hb.oppPairs.data();
    for (size_t index = start; index < end; index++) {
      if (fabsf(integrals[index]) < epsilon) break;
      int a = 2 * orbIndices[2 * index] + closed[i] % 2;
      int b = 2 * orbIndices[2 * index + 1] + closed[j] % 2;
      if (!restr_two(rs, closed[i], closed[j], a, b)) continue;
      if (!(getocc(d, a) || getocc(d, b))) {
        PtStochCand c;
        c.d = d;
        setocc(c.d, a, true);
        setocc(c.d, b, true);
        setocc(c.d, closed[i], false);
        setocc(c.d, closed[j], false);
        double sgn = pt_double_sign(c.d, a, b, closed[i], closed[j]);
        c.num1 = integrals[index] * sgn * ci1;
        c.num2 = integrals[index] * integrals[index] * ci1 * (ci1 * Nmcd / (Nmcd - 1) - ci2);
        c.E = energy_after_double(I, closed, nclosed, i, a, j, b, Energyd);
        c.present = fabs(integrals[index]) > epsilonLarge;
        out.push_back(c);
      }
    }
  }
}

// Uniform [0, 1) from a 64-bit Mersenne twister (the reference draws
// rand() / RAND_MAX from the C library; any uniform stream gives the same
// estimator, and this one is the same on every platform).
struct PtRng {
  std::mt19937_64 g;
  explicit PtRng(uint64_t seed) : g(seed) {}
  double next() { return (double)(g() >> 11) * (1.0 / 9007199254740992.0); }
};

// SHCIsampledeterminants::setUpAliasMethod (SHCI/SHCIsampledeterminants.cpp:64-88).
static void alias_setup(const double* ci, size_t N, double cumulative, std::vector<int>& alias,
                        std::vector<double>& prob) {
  alias.assign(N, 0);
  prob.assign(N, 0.0);
  std::vector<int> larger, smaller;
  for (size_t i = 0; i < N; i++) {
    prob[i] = fabs(ci[i]) * N / cumulative;
    if (prob[i] < 1.0)
      smaller.push_back((int)i);
    else
      larger.push_back((int)i);
  }
  while (!larger.empty() && !smaller.empty()) {
    int l = larger.back();
    larger.pop_back();
    int s_ = smaller.back();
    smaller.pop_back();
    alias[s_] = l;
    prob[l] = prob[l] - (1.0 - prob[s_]);
    if (prob[l] < 1.0)
      smaller.push_back(l);
    else
      larger.push_back(l);
  }
}

// SHCIsampledeterminants::sample_N2_alias (SHCI/SHCIsampledeterminants.cpp:153-190):
// Nmc draws, distinct determinants in order of first draw, weights
// cumulative * sign(c) summed over repeated draws, divided by Nmc.
static int alias_sample(const double* ci, size_t N, double cumulative, const std::vector<int>& alias,
                        const std::vector<double>& prob, int Nmc, PtRng& rng, std::vector<int>& sample,
                        std::vector<double>& wts) {
  sample.assign(Nmc, -1);
  wts.assign(Nmc, 0.0);
  int n = 0;
  for (int k = 0; k < Nmc; k++) {
    int det = (int)floor(rng.next() * N);
    if (rng.next() >= prob[det]) det = alias[det];
    int at = -1;
    for (int q = 0; q < n; ++q)
      if (sample[q] == det) {
        at = q;
        break;
      }
    const double w = cumulative * ci[det] / fabs(ci[det]);
    if (at < 0) {
      sample[n] = det;
      wts[n] = w;
      n++;
    } else {
      wts[at] += w;
    }
  }
  for (int k = 0; k < Nmc; k++) wts[k] /= Nmc;
  return n;
}

struct PtStochStats {
  int iterations = 0;
  double stddev = 0.0;
  double e_large = 0.0;  // the deterministic part at epsilon2Large
};

// SHCIbasics::DoPerturbativeStochastic2SingleListDoubleEpsilon2AllTogether
// (SHCI/SHCIbasics.cpp:55-451), one rank: the deterministic part at
// epsilon2Large (when below 999), then iterations of Nsample alias draws with
// probability |c_i| / sum |c|; each iteration's estimate is
// -sum_a (N1a^2 Nmc/(Nmc-1) - N2a) / (E_a - E0) over determinants outside the
// variational space, plus the same sum restricted to the contributions above
// epsilon2Large, plus the deterministic part. Stops once the standard error
// of the mean (from the fifth iteration on) is below targetError, or after
// nPTiter iterations. Returns the mean (the reference returns the running sum
// if nPTiter runs out first).
static double pt_semistochastic(const Ints& I, const HeatBath& hb, const Det* dets, size_t N, const double* ci,
                                double E0, double eps2, double eps2Large, int Nsample, int nPTiter,
                                double targetError, uint64_t seed, std::vector<Restriction> rs,
                                PtStochStats& st) {
  st = PtStochStats();
  if (eps2Large < 999) {
    PtStats dst;
    st.e_large = pt_deterministic(I, hb, dets, N, ci, E0, eps2Large, rs, dst);
  }
  double cumulative = 0.0;
  for (size_t i = 0; i < N; i++) cumulative += fabs(ci[i]);
  std::vector<int> alias;
  std::vector<double> prob;
  alias_setup(ci, N, cumulative, alias, prob);
  std::vector<Det> sorted(dets, dets + N);
  std::sort(sorted.begin(), sorted.end(), det_less);
  PtRng rng(seed);
  const int Nmc = Nsample;
  double avg = 0.0, avg2 = 0.0;
  std::vector<int> sample;
  std::vector<double> wts;
  std::vector<PtStochCand> all;
  for (int iter = 0; iter < nPTiter; iter++) {
    const int distinct = alias_sample(ci, N, cumulative, alias, prob, Nmc, rng, sample, wts);
    all.clear();
    for (int k = 0; k < distinct; k++) {
      const int Id = sample[k];
      pt_stoch_from_parent(I, hb, dets[Id], eps2 / fabs(ci[Id]), eps2Large / fabs(ci[Id]), wts[k], ci[Id], Nmc, rs,
                           all);
    }
    std::stable_sort(all.begin(), all.end(),
                     [](const PtStochCand& x, const PtStochCand& y) { return det_less(x.d, y.d); });
    double eA = 0.0, eB = 0.0;
    size_t k = 0, v = 0;
    const double f = 1. * Nmc / (Nmc - 1);
    while (k < all.size()) {
      size_t e = k;
      double n1a = 0, n2a = 0, n1b = 0, n2b = 0;
      while (e < all.size() && det_eq(all[e].d, all[k].d)) {
        n1a += all[e].num1;
        n2a += all[e].num2;
        if (all[e].present) {
          n1b += all[e].num1;
          n2b += all[e].num2;
        }
        ++e;
      }
      while (v < sorted.size() && det_less(sorted[v], all[k].d)) ++v;
      const bool in_space = v < sorted.size() && det_eq(sorted[v], all[k].d);
      if (!in_space) {
        const double de = all[k].E - E0;
        eA += (pow(fabs(n1a), 2) * f - n2a) / de;
        eB += (pow(fabs(n1b), 2) * f - n2b) / de;
      }
      k = e;
    }
    const double est = -eA + eB + st.e_large;
    avg += est;
    avg2 += est * est;
    const int it = iter + 1;
    st.iterations = it;
    st.stddev = it < 5 ? 1e4 : pow((it * avg2 - pow(avg, 2)) / it / (it - 1) / it, 0.5);
    if (st.stddev < targetError) break;
  }
  return avg / st.iterations;
}

// ---------------------------------------------------------------------------
// Reduced density matrices of the variational wavefunction
// ---------------------------------------------------------------------------
// SHCIrdm::populateSpatialRDM (SHCI/SHCIrdm.cpp:846-861): s2 is the n^2 x n^2
// spatial 2-RDM, element (I n + J, K n + L) at (I n + J) n^2 + K n + L.
static void populate_spatial(std::vector<double>& s2, int n, int i, int j, int k, int l, double v) {
  const size_t n2 = (size_t)n * n;
  const int I = i / 2, J = j / 2, K = k / 2, L = l / 2;
  if (i % 2 == l % 2 && j % 2 == k % 2) {
    s2[(size_t)(I * n + J) * n2 + L * n + K] -= v;
    s2[(size_t)(J * n + I) * n2 + K * n + L] -= v;
  }
  if (i % 2 == k % 2 && l % 2 == j % 2) {
    s2[(size_t)(I * n + J) * n2 + K * n + L] += v;
    s2[(size_t)(J * n + I) * n2 + L * n + K] += v;
  }
}

// getOrbDiff(bra, ket) (SHCI/Determinants.cpp:508-560): spin orbitals created
// (occupied in bra only) and destroyed (in ket only), each ascending.
static int orb_diff(const Det& bra, const Det& ket, int* cre, int* des) {
  int nc = 0, nd = 0;
  for (int w = 0; w < W; ++w) {
    uint64_t u = bra.w[w] ^ ket.w[w];
    uint64_t b = u & bra.w[w], k = u & ket.w[w];
    while (b) {
      if (nc < 2) cre[nc] = __builtin_ctzll(b) + 64 * w;
      ++nc;
      b &= b - 1;
    }
    while (k) {
      if (nd < 2) des[nd] = __builtin_ctzll(k) + 64 * w;
      ++nd;
      k &= k - 1;
    }
  }
  return nc;
}

// SHCIrdm::EvaluateRDM (SHCI/SHCIrdm.cpp:863-993) and EvaluateOneRDM
// (:996-1100) with cibra = ciket = c, over the connection lists of the
// variational Hamiltonian (row i: the diagonal, then every connected J < i;
// orbital differences of getOrbDiff(Dets[J], Dets[i]), as the build stores
// them at SHCI/SHCImakeHamiltonian.cpp:578-588). s1 is the n x n spatial 1-RDM.
static void evaluate_rdm(const Ints& I, const Det* dets, const SparseHam& H, size_t N, const double* c,
                         std::vector<double>& s2, std::vector<double>& s1) {
  const int n = I.norb, nspin = 2 * n;
  s2.assign((size_t)n * n * n * n, 0.0);
  s1.assign((size_t)n * n, 0.0);
  int closed[128];
  for (size_t i = 0; i < N; i++) {
    const int nelec = closed_list(dets[i], nspin, closed);
    const double cii = c[i] * c[i];
    for (int n1 = 0; n1 < nelec; n1++)
      for (int n2 = 0; n2 < n1; n2++) populate_spatial(s2, n, closed[n1], closed[n2], closed[n1], closed[n2], cii);
    for (int n1 = 0; n1 < nelec; n1++) s1[(size_t)(closed[n1] / 2) * n + closed[n1] / 2] += cii;
    for (int64_t p = H.rowptr[i] + 1; p < H.rowptr[i + 1]; ++p) {
      const int J = H.col[p];
      int cre[2], des[2];
      const int nc = orb_diff(dets[J], dets[i], cre, des);
      const double w = c[J] * c[i];
      if (nc == 1) {
        const int c0 = cre[0], d0 = des[0];
        const double sgn0 = parity_between(dets[i], std::min(d0, c0), std::max(d0, c0));
        for (int n1 = 0; n1 < nelec; n1++) {
          const int k = closed[n1];
          if (k == d0 || k == c0) continue;
          const int a = std::max(k, c0), b = std::min(k, c0), II = std::max(k, d0), JJ = std::min(k, d0);
          double sgn = sgn0;
          if (!((k > c0 && k > d0) || (k < c0 && k < d0))) sgn *= -1.;
          populate_spatial(s2, n, a, b, II, JJ, sgn * w);
          populate_spatial(s2, n, II, JJ, a, b, sgn * w);
        }
        s1[(size_t)(c0 / 2) * n + d0 / 2] += sgn0 * w;
        s1[(size_t)(d0 / 2) * n + c0 / 2] += sgn0 * w;
      } else if (nc == 2) {
        const int c0 = cre[0], c1 = cre[1], d0 = des[0], d1 = des[1];
        // Determinant::parity(d1, d0, c1, c0, sgn) (SHCI/Determinants.cpp:332-357)
        Det t = dets[i];
        double sgn = parity_between(t, std::min(d1, c1), std::max(d1, c1));
        setocc(t, d1, false);
        setocc(t, c1, true);
        sgn *= parity_between(t, std::min(d0, c0), std::max(d0, c0));
        populate_spatial(s2, n, c1, c0, d1, d0, sgn * w);
        populate_spatial(s2, n, d1, d0, c1, c0, sgn * w);
      }
    }
  }
}

// SHCIrdm::ComputeEnergyFromSpatialRDM (SHCI/SHCIrdm.cpp:1188-1245).
static double rdm_energy(const Ints& I, const std::vector<double>& s2, int nelec) {
  const int n = I.norb;
  const size_t n2 = (size_t)n * n;
  std::vector<double> one(n2, 0.0);
  for (int p = 0; p < n; p++)
    for (int q = 0; q < n; q++)
      for (int r = 0; r < n; r++) one[p * n + q] += s2[(size_t)(p * n + r) * n2 + q * n + r] / (1. * nelec - 1.);
  double onebody = 0.0, twobody = 0.0;
  for (int p = 0; p < n; p++)
    for (int q = 0; q < n; q++) onebody += I.i1(2 * p, 2 * q) * one[p * n + q];
  for (int p = 0; p < n; p++)
    for (int q = 0; q < n; q++)
      for (int r = 0; r < n; r++)
        for (int s_ = 0; s_ < n; s_++)
          twobody += 0.5 * s2[(size_t)(p * n + q) * n2 + r * n + s_] * I.i2(2 * p, 2 * r, 2 * q, 2 * s_);
  return I.coreE + onebody + twobody;
}

// Hmult2::operator() (SHCI/Hmult.h:52-150), serial branch: symmetric
// scatter from the lower triangle.
static void sigma(const SparseHam& H, size_t N, const double* x, double* y) {
  std::vector<double> yt(N, 0.0);
  for (size_t i = 0; i < N; i++) {
    for (int64_t p = H.rowptr[i]; p < H.rowptr[i + 1]; ++p) {
      double h = H.val[p];
      int J = H.col[p];
      yt[i] += h * x[J];
      if ((size_t)J != i) yt[J] += h * x[i];
    }
  }
  for (size_t j = 0; j < N; j++) y[j] = yt[j];
}

// Hmult2::operator() (SHCI/Hmult.h:52-150), parallel branch for fewer than
// 1e8 determinants: worker w of T owns the rows i with i % T == w (the
// reference's MPI ranks own every size-th row), scatters symmetrically into a
// private full-length ytemp, and the T vectors are summed in worker order (the
// reference's MPI_Reduce into local rank 0). Threads stand in for the ranks of
// one node.
static void sigma_mt(const SparseHam& H, size_t N, const double* x, double* y, int T) {
  if (T < 1) T = 1;
  std::vector<std::vector<double>> yt(T);
  std::vector<std::thread> pool;
  for (int w = 0; w < T; ++w)
    pool.emplace_back([&, w] {
      std::vector<double>& t = yt[w];
      t.assign(N, 0.0);
      for (size_t i = (size_t)w; i < N; i += (size_t)T)
        for (int64_t p = H.rowptr[i]; p < H.rowptr[i + 1]; ++p) {
          const double h = H.val[p];
          const int J = H.col[p];
          t[i] += h * x[J];
          if ((size_t)J != i) t[J] += h * x[i];
        }
    });
  for (auto& th : pool) th.join();
  // reduction, also split over the workers by ranges of the vector
  pool.clear();
  const size_t chunk = (N + T - 1) / T;
  for (int w = 0; w < T; ++w)
    pool.emplace_back([&, w] {
      const size_t a = std::min(N, (size_t)w * chunk), b = std::min(N, a + chunk);
      for (size_t j = a; j < b; ++j) {
        double v = 0.0;
        for (int r = 0; r < T; ++r) v += yt[r][j];
        y[j] = v;
      }
    });
  for (auto& th : pool) th.join();
}

// ---------------------------------------------------------------------------
// Dense symmetric eigensolver (cyclic Jacobi) for the Davidson subspace. The
// reference uses Eigen::SelfAdjointEigenSolver (SHCI/Davidson.cpp:262); both
// return ascending eigenvalues with orthonormal eigenvectors.
// ---------------------------------------------------------------------------
static void jacobi_eig(int m, std::vector<double> A, std::vector<double>& evals, std::vector<double>& evecs) {
  // A row-major m x m symmetric; evecs column-major m x m (column k = vector k)
  std::vector<double> V((size_t)m * m, 0.0);
  for (int i = 0; i < m; ++i) V[(size_t)i * m + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < m; ++p)
      for (int q = p + 1; q < m; ++q) off += A[(size_t)p * m + q] * A[(size_t)p * m + q];
    if (off < 1e-300) break;
    for (int p = 0; p < m; ++p)
      for (int q = p + 1; q < m; ++q) {
        double apq = A[(size_t)p * m + q];
        if (fabs(apq) < 1e-300) continue;
        double app = A[(size_t)p * m + p], aqq = A[(size_t)q * m + q];
        double theta = (aqq - app) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < m; ++k) {
          double akp = A[(size_t)k * m + p], akq = A[(size_t)k * m + q];
          A[(size_t)k * m + p] = c * akp - s * akq;
          A[(size_t)k * m + q] = s * akp + c * akq;
        }
        for (int k = 0; k < m; ++k) {
          double apk = A[(size_t)p * m + k], aqk = A[(size_t)q * m + k];
          A[(size_t)p * m + k] = c * apk - s * aqk;
          A[(size_t)q * m + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < m; ++k) {
          double vkp = V[(size_t)k * m + p], vkq = V[(size_t)k * m + q];
          V[(size_t)k * m + p] = c * vkp - s * vkq;
          V[(size_t)k * m + q] = s * vkp + c * vkq;
        }
      }
  }
  std::vector<int> ord(m);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return A[(size_t)x * m + x] < A[(size_t)y * m + y]; });
  evals.resize(m);
  evecs.assign((size_t)m * m, 0.0);
  for (int k = 0; k < m; ++k) {
    evals[k] = A[(size_t)ord[k] * m + ord[k]];
    for (int i = 0; i < m; ++i) evecs[(size_t)k * m + i] = V[(size_t)i * m + ord[k]];
  }
}

static double dot(const double* a, const double* b, size_t n) {
  double s = 0.0;
  for (size_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

// Deterministic stand-in for Eigen's setRandom (uniform in [-1,1]); the
// reference seeds it from the clock unless `seed` is given.
static uint64_t g_rng = 0x9E3779B97F4A7C15ull;
static double rnd_pm1() {
  g_rng ^= g_rng << 13;
  g_rng ^= g_rng >> 7;
  g_rng ^= g_rng << 17;
  return ((g_rng >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0;
}

// davidson / davidsonDirect (SHCI/Davidson.cpp:111-348, :353-590) and
// precondition (:85-106). `direct` selects davidsonDirect's collapse rule and
// iteration cap. Returns 0 on success, 1 on non-convergence.
static int davidson(const SparseHam& H, size_t N, std::vector<std::vector<double>>& x0,
                    const std::vector<double>& diag, int maxCopies, double tol, bool direct,
                    std::vector<double>& eroots, int& numIter) {
  const int nroots = (int)x0.size();
  eroots.clear();
  std::vector<std::vector<double>> b(maxCopies, std::vector<double>(N, 0.0));
  std::vector<std::vector<double>> sig(maxCopies, std::vector<double>(N, 0.0));
  for (int i = 0; i < nroots; i++) {
    b[i] = x0[i];
    if (sqrt(dot(x0[i].data(), x0[i].data(), N)) < 1.e-10) {
      for (size_t k = 0; k < N; ++k) b[i][k] = rnd_pm1();
      double nn = sqrt(dot(b[i].data(), b[i].data(), N));
      for (size_t k = 0; k < N; ++k) b[i][k] /= nn;
    }
  }
  for (int i = 0; i < nroots; i++) {
    for (int j = 0; j < i; j++) {
      double ov = dot(b[j].data(), b[i].data(), N);
      for (size_t k = 0; k < N; ++k) b[i][k] -= ov * b[j][k];
    }
    if (sqrt(dot(b[i].data(), b[i].data(), N)) < 1e-8)
      for (size_t k = 0; k < N; ++k) b[i][k] = rnd_pm1();
    for (int j = 0; j < i; j++) {
      double ov = dot(b[j].data(), b[i].data(), N);
      for (size_t k = 0; k < N; ++k) b[i][k] -= ov * b[j][k];
    }
    double nn = sqrt(dot(b[i].data(), b[i].data(), N));
    for (size_t k = 0; k < N; ++k) b[i][k] /= nn;
  }
  int sigmaSize = 0, bsize = nroots;
  std::vector<double> r(N);
  int convergedRoot = 0;
  numIter = 0;
  double ei = 0.0;
  std::vector<double> tmp;
  while (true) {
    for (int i = sigmaSize; i < bsize; i++) {
      if (g_threads > 1)
        sigma_mt(H, N, b[i].data(), sig[i].data(), g_threads);
      else
        sigma(H, N, b[i].data(), sig[i].data());
      sigmaSize++;
    }
    std::vector<double> hs((size_t)bsize * bsize);
    for (int i = 0; i < bsize; i++)
      for (int j = i; j < bsize; j++) {
        hs[(size_t)i * bsize + j] = dot(b[i].data(), sig[j].data(), N);
        hs[(size_t)j * bsize + i] = hs[(size_t)i * bsize + j];
      }
    std::vector<double> ev, evec;
    jacobi_eig(bsize, hs, ev, evec);
    // b <- b * V ; sigma <- sigma * V
    tmp.assign((size_t)bsize * N, 0.0);
    for (int kcol = 0; kcol < bsize; ++kcol)
      for (int i = 0; i < bsize; ++i) {
        double c = evec[(size_t)kcol * bsize + i];
        const double* src = b[i].data();
        double* dst = &tmp[(size_t)kcol * N];
        for (size_t k = 0; k < N; ++k) dst[k] += c * src[k];
      }
    for (int kcol = 0; kcol < bsize; ++kcol) std::copy(&tmp[(size_t)kcol * N], &tmp[(size_t)kcol * N] + N, b[kcol].begin());
    tmp.assign((size_t)bsize * N, 0.0);
    for (int kcol = 0; kcol < bsize; ++kcol)
      for (int i = 0; i < bsize; ++i) {
        double c = evec[(size_t)kcol * bsize + i];
        const double* src = sig[i].data();
        double* dst = &tmp[(size_t)kcol * N];
        for (size_t k = 0; k < N; ++k) dst[k] += c * src[k];
      }
    for (int kcol = 0; kcol < bsize; ++kcol) std::copy(&tmp[(size_t)kcol * N], &tmp[(size_t)kcol * N] + N, sig[kcol].begin());

    ei = ev[convergedRoot];
    for (int i = 0; i < convergedRoot; i++) {
      for (size_t k = 0; k < N; ++k) r[k] = sig[i][k] - ev[i] * b[i][k];
      double error = sqrt(dot(r.data(), r.data(), N));
      if (error > tol) convergedRoot = i;
    }
    for (size_t k = 0; k < N; ++k) r[k] = sig[convergedRoot][k] - ei * b[convergedRoot][k];
    double error = sqrt(dot(r.data(), r.data(), N));
    numIter++;
    if ((size_t)bsize == N) {
      for (int i = 0; i < nroots; i++) {
        x0[i] = b[i];
        eroots.push_back(ev[i]);
      }
      return 0;
    }
    const int cap = direct ? 400 * nroots : 800 * nroots;
    if (error < tol || numIter > cap) {
      if (numIter > (direct ? 400 * nroots : 2000 * nroots)) return 1;
      convergedRoot++;
      if (convergedRoot == nroots) {
        for (int i = 0; i < convergedRoot; i++) {
          x0[i] = b[i];
          eroots.push_back(ev[i]);
        }
        return 0;
      }
    }
    for (size_t k = 0; k < N; ++k) {
      if (fabs(ei - diag[k]) > 1e-12)
        r[k] = r[k] / (ei - diag[k]);
      else
        r[k] = r[k] / (ei - diag[k] - 1.e-12);
    }
    for (int i = 0; i < bsize; i++) {
      double ov = dot(b[i].data(), r.data(), N) / dot(b[i].data(), b[i].data(), N);
      for (size_t k = 0; k < N; ++k) r[k] -= ov * b[i][k];
    }
    double rn = sqrt(dot(r.data(), r.data(), N));
    if (bsize < maxCopies) {
      for (size_t k = 0; k < N; ++k) b[bsize][k] = r[k] / rn;
      bsize++;
    } else {
      if (direct) {
        bsize = std::min(nroots + 3, maxCopies);
        sigmaSize = bsize - 1;
      } else {
        bsize = nroots + 3;
        sigmaSize = nroots + 2;
      }
      for (size_t k = 0; k < N; ++k) b[bsize - 1][k] = r[k] / rn;
    }
  }
}

// ---------------------------------------------------------------------------
// input.dat (SHCI/input.cpp:35-404), variational subset.
// ---------------------------------------------------------------------------
struct Schedule {
  std::vector<std::vector<int>> occupied;
  std::vector<double> epsilon1;
  int nroots = 1;
  double davidsonTol = 5e-5, davidsonTolLoose = 5e-5, dE = 1e-8;
  bool direct = false;
  SelParams sel;
  std::string integralFile = "FCIDUMP";
  double epsilon2 = 1.e-8;  // SHCI/input.cpp:58
  bool stochastic = true;   // SHCI/input.cpp:67; `deterministic` clears it (:322-323)
};

static int read_input(const char* path, Schedule& s, std::string& err) {
  std::ifstream ifs(path);
  if (!ifs.good()) {
    err = std::string("cannot open ") + path;
    return 1;
  }
  std::stringstream dump;
  dump << ifs.rdbuf();
  int maxiter = -1, nocc = -1;
  std::vector<int> sweep_iter;
  std::vector<double> sweep_eps;
  std::vector<std::string> tok;
  while (dump.good()) {
    std::string Line;
    std::getline(dump, Line);
    split_compress(Line, ", \t\n", tok);
    std::string arg = tok[0];
    if (arg.empty() || arg[0] == '#') continue;
    if (iequals(arg, "nocc")) {
      nocc = atoi(tok[1].c_str());
      std::getline(dump, Line);
      split_compress(Line, ", \t", tok);
      while (!iequals(tok[0], "end")) {
        if ((int)tok.size() != nocc) {
          err = "nocc count mismatch";
          return 2;
        }
        std::vector<int> occ;
        for (auto& t : tok) occ.push_back(atoi(t.c_str()));
        s.occupied.push_back(occ);
        std::getline(dump, Line);
        split_compress(Line, ", \t", tok);
      }
    } else if (iequals(arg, "nact")) s.sel.nact = atoi(tok[1].c_str());
    else if (iequals(arg, "ncore")) s.sel.ncore = atoi(tok[1].c_str());
    else if (iequals(arg, "directdavidson")) s.direct = true;
    else if (iequals(arg, "nroots")) s.nroots = (int)atof(tok[1].c_str());
    else if (iequals(arg, "orbitals")) s.integralFile = tok[1];
    else if (iequals(arg, "davidsonTol")) s.davidsonTol = atof(tok[1].c_str());
    else if (iequals(arg, "davidsonTolLoose")) s.davidsonTolLoose = atof(tok[1].c_str());
    else if (iequals(arg, "dE")) s.dE = atof(tok[1].c_str());
    else if (iequals(arg, "maxiter")) maxiter = atoi(tok[1].c_str());
    else if (iequals(arg, "epsilon2")) s.epsilon2 = atof(tok[1].c_str());
    else if (iequals(arg, "deterministic")) s.stochastic = false;
    else if (iequals(arg, "restrict") || iequals(arg, "restrictv")) {
      Restriction r;
      r.minElec = atoi(tok[1].c_str());
      r.maxElec = atoi(tok[2].c_str());
      for (size_t i = 3; i < tok.size(); i++) {
        r.orbs.push_back(2 * atoi(tok[i].c_str()));
        r.orbs.push_back(2 * atoi(tok[i].c_str()) + 1);
      }
      s.sel.restrictions.push_back(r);
    } else if (iequals(arg, "schedule")) {
      std::getline(dump, Line);
      std::vector<std::string> st;
      split_compress(Line, " \t", st);
      while (!iequals(st[0], "END")) {
        if (st[0].empty() || st[0][0] != '#') {
          sweep_iter.push_back(atoi(st[0].c_str()));
          sweep_eps.push_back(atof(st.size() > 1 ? st[1].c_str() : "0"));
        }
        if (!dump.good()) break;
        std::getline(dump, Line);
        split_compress(Line, " \t", st);
      }
    }
    // every other keyword belongs to stages outside the variational path
  }
  if (sweep_iter.empty() || maxiter < sweep_iter.back()) {
    err = "maxiter should be greater than last entry of sweep_iter";
    return 3;
  }
  if (nocc == -1) {
    err = "nocc keyword has to be included.";
    return 4;
  }
  if (s.direct) s.davidsonTolLoose = 3.e-2;
  for (size_t i = 1; i < sweep_iter.size(); i++)
    for (int j = sweep_iter[i - 1]; j < sweep_iter[i]; j++) s.epsilon1.push_back(sweep_eps[i - 1]);
  for (int j = sweep_iter.back(); j < maxiter; j++) s.epsilon1.push_back(sweep_eps.back());
  return 0;
}

// ---------------------------------------------------------------------------
// Variational driver: SHCI/SHCI.cpp:289-427 (reference dets, initial ci) and
// SHCIbasics::DoVariational (SHCI/SHCIbasics.cpp:783-1378), serial, no Trev,
// no restart files.
// ---------------------------------------------------------------------------
struct IterLog {
  int iter;
  double eps1;
  int64_t ndets;
  double energy;  // root 0, coreE added
  int davidson_iters;
  double seconds;
};
struct VarResult {
  std::vector<double> E;  // per root, coreE added
  std::vector<Det> dets;  // final variational space, in index order
  std::vector<std::vector<double>> ci;
  std::vector<IterLog> log;
  int64_t nnz_lower = 0;
  double seconds = 0.0;
  SparseHam H;  // the final space's lower triangle (kept for timing its sigma)
};

static double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

static int do_variational(const Ints& I, const HeatBath& hb, Schedule& s, VarResult& res, std::string& err,
                          int verbose) {
  double t0 = now_s();
  // reference dets and initial ci (SHCI/SHCI.cpp:289-399)
  std::vector<Det> Dets(s.occupied.size());
  int lowest = 0;
  double lowestE = 1e12;
  for (size_t d = 0; d < s.occupied.size(); ++d) {
    memset(&Dets[d], 0, sizeof(Det));
    for (int p : s.occupied[d]) {
      if (p < 0 || p >= 2 * I.norb || getocc(Dets[d], p)) {
        err = "bad or repeated orbital in nocc";
        return 1;
      }
      setocc(Dets[d], p, true);
    }
    if ((int)s.occupied[d].size() != I.nelec) {
      err = "nocc differs from NELEC";
      return 2;
    }
    double E = det_energy(I, Dets[d]) + I.coreE;
    if (E < lowestE) {
      lowestE = E;
      lowest = (int)d;
    }
  }
  const int nroots = s.nroots;
  std::vector<std::vector<double>> ci(nroots, std::vector<double>(Dets.size(), 0.0));
  for (size_t j = 0; j < Dets.size(); ++j) ci[0][j] = 1.0;
  ci[0][lowest] += Dets.size();
  double nn = sqrt(dot(ci[0].data(), ci[0].data(), Dets.size()));
  for (auto& v : ci[0]) v /= nn;

  std::vector<Det> sorted = Dets;
  std::sort(sorted.begin(), sorted.end(), det_less);
  std::vector<double> diag;
  std::vector<double> E0(nroots, fabs(det_energy(I, Dets[0])));
  SparseHam H;
  for (size_t iter = 0; iter < s.epsilon1.size(); ++iter) {
    double eps1 = s.epsilon1[iter];
    size_t N0 = Dets.size();
    std::vector<double> cMax(N0, 0.0);
    for (size_t j = 0; j < N0; j++) {
      for (int i = 0; i < nroots; i++) cMax[j] += pow(fabs(ci[i][j]), 2);
      cMax[j] = pow(cMax[j], 0.5);
    }
    std::vector<Det> newDets;
    const double ts0 = now_s();
    select_all(I, hb, Dets.data(), N0, cMax.data(), eps1, s.sel, sorted.data(), sorted.size(), newDets);
    const double ts1 = now_s();
    std::vector<std::vector<double>> X0(nroots, std::vector<double>(N0 + newDets.size(), 0.0));
    for (int i = 0; i < nroots; i++) std::copy(ci[i].begin(), ci[i].end(), X0[i].begin());
    Dets.insert(Dets.end(), newDets.begin(), newDets.end());
    size_t N = Dets.size();
    build_ham(I, Dets.data(), N, H, N0);  // the rows of the first N0 determinants are kept
    const double ts2 = now_s();
    sorted = Dets;
    std::sort(sorted.begin(), sorted.end(), det_less);
    size_t old = diag.size();
    diag.resize(N);
    for (size_t k = old; k < N; ++k) diag[k] = det_energy(I, Dets[k]);
    double prevE0 = (iter == 0) ? -10.0 : E0[0];
    int numIter = 0;
    std::vector<double> ev;
    int rc = davidson(H, N, X0, diag, s.direct ? nroots + 2 : nroots + 4, s.davidsonTolLoose, s.direct, ev,
                      numIter);
    if (rc) {
      err = "Davidson calculation did not converge";
      return 3;
    }
    E0 = ev;
    ci = X0;
    res.log.push_back({(int)iter, eps1, (int64_t)N, E0[0] + I.coreE, numIter, now_s() - t0});
    if (verbose > 1)
      fprintf(stderr, "[oracle] iter %d: select %.2f s, build %.2f s (%zu lower-triangle entries), davidson %.2f s\n",
              (int)iter, ts1 - ts0, ts2 - ts1, H.col.size(), now_s() - ts2);
    if (verbose)
      printf("%4d %4d  %10.2e  %10zu   %18.10f  %9d  %10.2f\n", (int)iter, 0, eps1, N, E0[0] + I.coreE, numIter,
             now_s() - t0);
    if (fabs(E0[0] - prevE0) < s.dE || iter == s.epsilon1.size() - 1) {
      rc = davidson(H, N, ci, diag, nroots + 4, s.davidsonTol, s.direct, ev, numIter);
      if (rc) {
        err = "Davidson calculation did not converge";
        return 3;
      }
      E0 = ev;
      break;
    }
  }
  res.E.resize(nroots);
  for (int i = 0; i < nroots; ++i) res.E[i] = E0[i] + I.coreE;
  res.dets = Dets;
  res.ci = ci;
  res.nnz_lower = H.col.size();
  res.H = std::move(H);
  res.seconds = now_s() - t0;
  return 0;
}

}  // namespace orc

// ===========================================================================
// C interface used by the Python test harness (oracle/oracle.py).
// ===========================================================================
using namespace orc;

struct orc_ctx {
  Ints ints;
  HeatBath hb;
  SparseHam ham;
  size_t ham_n = 0;
  std::vector<Det> ham_dets;  // the space of the last orc_ham_build
  VarResult var;
  Schedule sched;
  PtStats pt;
  std::string err;
};

static std::vector<Restriction> unpack_restrictions(const int64_t* restr, int nrestr) {
  std::vector<Restriction> rs;
  for (int r = 0; r < nrestr; ++r) {
    Restriction R;
    R.minElec = (int)restr[4 * r];
    R.maxElec = (int)restr[4 * r + 1];
    uint64_t m0 = (uint64_t)restr[4 * r + 2];
    for (int k = 0; k < 64; ++k)
      if ((m0 >> k) & 1) {
        R.orbs.push_back(2 * k);
        R.orbs.push_back(2 * k + 1);
      }
    rs.push_back(R);
  }
  return rs;
}

extern "C" {

const char* orc_last_error(orc_ctx* c) { return c ? c->err.c_str() : "null context"; }

orc_ctx* orc_load(const char* fcidump, char* errbuf, int errlen) {
  orc_ctx* c = new orc_ctx();
  std::string err;
  if (read_fcidump(fcidump, c->ints, err)) {
    if (errbuf && errlen > 0) snprintf(errbuf, errlen, "%s", err.c_str());
    delete c;
    return nullptr;
  }
  build_heatbath(c->ints, c->hb);
  return c;
}

void orc_free(orc_ctx* c) { delete c; }

void orc_info(orc_ctx* c, int* norb, int* nelec, double* coreE, double* maxEntry) {
  *norb = c->ints.norb;
  *nelec = c->ints.nelec;
  *coreE = c->ints.coreE;
  *maxEntry = c->ints.maxEntry;
}

// packed integrals, for cross-checking the GPU library's reader
int64_t orc_i2_size(orc_ctx* c) { return (int64_t)c->ints.I2.size(); }
void orc_i2_export(orc_ctx* c, double* out) { std::copy(c->ints.I2.begin(), c->ints.I2.end(), out); }
void orc_i1_export(orc_ctx* c, double* out) { std::copy(c->ints.I1.begin(), c->ints.I1.end(), out); }

int64_t orc_hb_size(orc_ctx* c, int same) { return same ? c->hb.sameVal.size() : c->hb.oppVal.size(); }
void orc_hb_export(orc_ctx* c, int same, float* vals, int16_t* pairs, uint64_t* starts, double* singles) {
  auto& V = same ? c->hb.sameVal : c->hb.oppVal;
  auto& P = same ? c->hb.samePairs : c->hb.oppPairs;
  auto& S = same ? c->hb.sameStart : c->hb.oppStart;
  if (vals) std::copy(V.begin(), V.end(), vals);
  if (pairs) std::copy(P.begin(), P.end(), pairs);
  if (starts) std::copy(S.begin(), S.end(), starts);
  if (singles) std::copy(c->hb.Singles.begin(), c->hb.Singles.end(), singles);
}

double orc_energy(orc_ctx* c, const uint64_t* det) {
  Det d;
  memcpy(&d, det, sizeof(Det));
  return det_energy(c->ints, d);
}

double orc_hij(orc_ctx* c, const uint64_t* bra, const uint64_t* ket) {
  Det b, k;
  memcpy(&b, bra, sizeof(Det));
  memcpy(&k, ket, sizeof(Det));
  return hij(c->ints, b, k);
}

// Selection from every parent with threshold eps1/|cmax_i|; candidates present
// in `existing` are dropped; result sorted and unique. restr: nrestr triples
// (min, max, spatial-orbital mask lo, hi) packed as int64[4].
int64_t orc_select(orc_ctx* c, const uint64_t* dets, int64_t n, const double* cmax, double eps1,
                   const uint64_t* existing_sorted, int64_t nexisting, int ncore, int nact,
                   const int64_t* restr, int nrestr, uint64_t* out, int64_t cap) {
  SelParams sp;
  sp.ncore = ncore;
  sp.nact = nact;
  sp.restrictions = unpack_restrictions(restr, nrestr);
  std::vector<Det> nd;
  select_all(c->ints, c->hb, (const Det*)dets, (size_t)n, cmax, eps1, sp, (const Det*)existing_sorted,
             (size_t)nexisting, nd);
  if ((int64_t)nd.size() <= cap) memcpy(out, nd.data(), nd.size() * sizeof(Det));
  return (int64_t)nd.size();
}

// Lower-triangle Hamiltonian with the diagonal first in every row (SparseHam).
// Builds the lower triangle of the space (every stride-th row when stride > 1,
// with orc_set_threads workers); returns the entries kept.
int64_t orc_ham_build_strided(orc_ctx* c, const uint64_t* dets, int64_t n, int64_t stride) {
  build_ham(c->ints, (const Det*)dets, (size_t)n, c->ham, 0, (size_t)std::max<int64_t>(1, stride));
  c->ham_n = (size_t)n;
  c->ham_dets.assign((const Det*)dets, (const Det*)dets + n);
  return (int64_t)c->ham.col.size();
}
int64_t orc_ham_build(orc_ctx* c, const uint64_t* dets, int64_t n) {
  build_ham(c->ints, (const Det*)dets, (size_t)n, c->ham);
  c->ham_n = (size_t)n;
  c->ham_dets.assign((const Det*)dets, (const Det*)dets + n);
  return (int64_t)c->ham.col.size();
}
void orc_ham_export(orc_ctx* c, int64_t* rowptr, int32_t* col, double* val) {
  std::copy(c->ham.rowptr.begin(), c->ham.rowptr.end(), rowptr);
  std::copy(c->ham.col.begin(), c->ham.col.end(), col);
  std::copy(c->ham.val.begin(), c->ham.val.end(), val);
}
void orc_sigma(orc_ctx* c, const double* x, double* y) { sigma(c->ham, c->ham_n, x, y); }
void orc_sigma_mt(orc_ctx* c, const double* x, double* y, int threads) {
  sigma_mt(c->ham, c->ham_n, x, y, threads);
}

// Dice's Davidson on the last built Hamiltonian. x0: nroots x n (row major);
// overwritten by the eigenvectors. Returns 0 or 1 (no convergence).
int orc_davidson(orc_ctx* c, double* x0, int nroots, const double* diag, int maxCopies, double tol, int direct,
                 double* eroots, int* numIter) {
  size_t n = c->ham_n;
  std::vector<std::vector<double>> X(nroots, std::vector<double>(n));
  for (int r = 0; r < nroots; ++r) std::copy(x0 + r * n, x0 + (r + 1) * n, X[r].begin());
  std::vector<double> d(diag, diag + n), ev;
  int rc = davidson(c->ham, n, X, d, maxCopies, tol, direct != 0, ev, *numIter);
  if (rc) return rc;
  for (int r = 0; r < nroots; ++r) {
    std::copy(X[r].begin(), X[r].end(), x0 + r * n);
    eroots[r] = ev[r];
  }
  return 0;
}

// Whole variational stage from a Dice input file. The FCIDUMP named in the
// input (or `fcidump_override`) is read relative to the current directory.
// Worker threads for selection, Hamiltonian rows and sigma (default 1: the
// serial restatement).
void orc_set_threads(int threads) { g_threads = threads < 1 ? 1 : threads; }

int orc_run_input(orc_ctx** out_ctx, const char* input, const char* fcidump_override, int verbose, char* errbuf,
                  int errlen) {
  Schedule s;
  std::string err;
  if (read_input(input, s, err)) {
    snprintf(errbuf, errlen, "%s", err.c_str());
    return 1;
  }
  const char* path = fcidump_override ? fcidump_override : s.integralFile.c_str();
  orc_ctx* c = orc_load(path, errbuf, errlen);
  if (!c) return 2;
  if (do_variational(c->ints, c->hb, s, c->var, err, verbose)) {
    snprintf(errbuf, errlen, "%s", err.c_str());
    delete c;
    return 3;
  }
  c->sched = s;
  // the run's Hamiltonian becomes the context's (orc_sigma / orc_sigma_mt)
  c->ham = std::move(c->var.H);
  c->ham_n = c->var.dets.size();
  *out_ctx = c;
  return 0;
}

// Deterministic PT2 correction for the given space and coefficients (E0 with
// coreE). restr as for orc_select (the PT restrictions). Returns E2.
double orc_pt_det(orc_ctx* c, const uint64_t* dets, int64_t n, const double* ci, double E0, double eps2,
                  const int64_t* restr, int nrestr) {
  return pt_deterministic(c->ints, c->hb, (const Det*)dets, (size_t)n, ci, E0, eps2,
                          unpack_restrictions(restr, nrestr), c->pt);
}
// The same with the candidates of parents [p0, p1) only.
double orc_pt_det_range(orc_ctx* c, const uint64_t* dets, int64_t n, const double* ci, double E0, double eps2,
                        int64_t p0, int64_t p1) {
  return pt_deterministic(c->ints, c->hb, (const Det*)dets, (size_t)n, ci, E0, eps2, {}, c->pt, (size_t)p0,
                          (size_t)p1);
}

// Spatial 2-RDM (n^4, element (p n + q, r n + s) at (p n + q) n^2 + r n + s)
// and spatial 1-RDM (n^2) of the wavefunction c on the space `dets`.
void orc_rdm(orc_ctx* c, const uint64_t* dets, int64_t n, const double* ci, double* s2, double* s1) {
  SparseHam H;
  build_ham(c->ints, (const Det*)dets, (size_t)n, H);
  std::vector<double> a, b;
  evaluate_rdm(c->ints, (const Det*)dets, H, (size_t)n, ci, a, b);
  std::copy(a.begin(), a.end(), s2);
  std::copy(b.begin(), b.end(), s1);
}
// The same on the space and connection lists of the last orc_ham_build
// (the evaluation alone, for timing).
void orc_rdm_eval(orc_ctx* c, const double* ci, double* s2, double* s1) {
  std::vector<double> a, b;
  evaluate_rdm(c->ints, c->ham_dets.data(), c->ham, c->ham_n, ci, a, b);
  std::copy(a.begin(), a.end(), s2);
  std::copy(b.begin(), b.end(), s1);
}
// Energy (coreE included) from a spatial 2-RDM.
double orc_rdm_energy(orc_ctx* c, const double* s2) {
  const size_t n4 = (size_t)c->ints.norb * c->ints.norb * c->ints.norb * c->ints.norb;
  return rdm_energy(c->ints, std::vector<double>(s2, s2 + n4), c->ints.nelec);
}

// PT2 on the result of orc_run_input for one root, eps2 <= 0 taking the
// input's epsilon2; the restrictions are the input's (`restrict` applies to
// both stages, SHCI/input.cpp:267-277). Returns E2.
double orc_var_pt(orc_ctx* c, int root, double eps2) {
  if (eps2 <= 0) eps2 = c->sched.epsilon2;
  return pt_deterministic(c->ints, c->hb, c->var.dets.data(), c->var.dets.size(), c->var.ci[root].data(),
                          c->var.E[root], eps2, c->sched.sel.restrictions, c->pt);
}
// Semistochastic PT2 of dets / ci (E0 with coreE). Returns E2; stats out.
double orc_pt_stoch(orc_ctx* c, const uint64_t* dets, int64_t n, const double* ci, double E0, double eps2,
                    double eps2Large, int Nsample, int nPTiter, double targetError, uint64_t seed, double* stddev,
                    int* iterations, double* e_large) {
  PtStochStats st;
  const double e2 = pt_semistochastic(c->ints, c->hb, (const Det*)dets, (size_t)n, ci, E0, eps2, eps2Large, Nsample,
                                      nPTiter, targetError, seed, c->sched.sel.restrictions, st);
  *stddev = st.stddev;
  *iterations = st.iterations;
  *e_large = st.e_large;
  return e2;
}
double orc_input_epsilon2(orc_ctx* c) { return c->sched.epsilon2; }
int orc_input_deterministic(orc_ctx* c) { return c->sched.stochastic ? 0 : 1; }
void orc_pt_stats(orc_ctx* c, int64_t* candidates, int64_t* unique, double* psi1_norm, int64_t* outside) {
  *outside = c->pt.outside;
  *candidates = c->pt.candidates;
  *unique = c->pt.unique;
  *psi1_norm = c->pt.psi1_norm;
}

int orc_var_nroots(orc_ctx* c) { return (int)c->var.E.size(); }
int64_t orc_var_ndets(orc_ctx* c) { return (int64_t)c->var.dets.size(); }
int orc_var_niters(orc_ctx* c) { return (int)c->var.log.size(); }
double orc_var_seconds(orc_ctx* c) { return c->var.seconds; }
int64_t orc_var_nnz_lower(orc_ctx* c) { return c->var.nnz_lower; }
void orc_var_energies(orc_ctx* c, double* E) { std::copy(c->var.E.begin(), c->var.E.end(), E); }
void orc_var_log(orc_ctx* c, int64_t* ndets, double* energy, int* dav_iters, double* eps1, double* secs) {
  for (size_t i = 0; i < c->var.log.size(); ++i) {
    ndets[i] = c->var.log[i].ndets;
    energy[i] = c->var.log[i].energy;
    dav_iters[i] = c->var.log[i].davidson_iters;
    eps1[i] = c->var.log[i].eps1;
    secs[i] = c->var.log[i].seconds;
  }
}
void orc_var_dets(orc_ctx* c, uint64_t* out) { memcpy(out, c->var.dets.data(), c->var.dets.size() * sizeof(Det)); }
void orc_var_ci(orc_ctx* c, int root, double* out) {
  std::copy(c->var.ci[root].begin(), c->var.ci[root].end(), out);
}

}  // extern "C"

#ifdef ORACLE_MAIN
int main(int argc, char** argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s input.dat [FCIDUMP]\n", argv[0]);
    return 1;
  }
  orc_ctx* c = nullptr;
  char err[512];
  int rc = orc_run_input(&c, argv[1], argc > 2 ? argv[2] : nullptr, 1, err, sizeof(err));
  if (rc) {
    fprintf(stderr, "error: %s\n", err);
    return rc;
  }
  for (size_t i = 0; i < c->var.E.size(); ++i) printf("root %zu  E_var %.12f\n", i, c->var.E[i]);
  if (!c->sched.stochastic)
    for (size_t i = 0; i < c->var.E.size(); ++i) {
      double e2 = orc_var_pt(c, (int)i, -1.0);
      printf("root %zu  E_PT2 %.12f  E_var+PT2 %.12f  candidates %lld unique %lld\n", i, e2, c->var.E[i] + e2,
             (long long)c->pt.candidates, (long long)c->pt.unique);
    }
  printf("ndets %zu  seconds %.3f\n", c->var.dets.size(), c->var.seconds);
  orc_free(c);
  return 0;
}
#endif

// Test infrastructure only: a CPU restatement of the BERTHA multi-centre
// Dirac-Coulomb Fock build (bertha-scf.f, CLMFAST and its callees).  Only
// tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py use it,
// as the checker; the GPU library never links or calls it.
//
// Parity status: the reference ships no golden vectors, and its Fortran
// cannot be compiled on this machine.  Its one recorded run, the YbF+
// Dirac-Coulomb SCF log, is the fixture tests/golden/ybf_plus_388.json.  The
// GPU SCF reproduces that log (tests/test_ybf_golden.py), and the GPU
// build matches this restatement to 1e-11 in the parity tests.  An SCF of
// the deck by this restatement's RACAH1-on route reaches the log's stage-3
// band (tests/golden/run_ybf_oracle_scf.py).  It is checked further against
// independent mathematics (tests/test_oracle_pins.py): Boys values against
// mpmath, the Hermite E-coefficients against direct evaluation of the
// spinor overlap densities, the time-reversal phase relations the reference
// relies on, and closed forms for (ss|ss).  It is also checked against the
// reference's one-centre Racah route (oracle/racah1.py,
// tests/test_oracle_racah1.py).
//
// Routines restated (bertha-scf.f line numbers):
//   FUNFM  32465-32619   Boys function, four regimes
//   RMAKE  31900-32462   Hermite R-integrals
//   EVRS/ESTEPLM/ESTEPL/ESTEPN 36981-37750  Saunders recursion
//   ESGTF  36900         Condon-Shortley phase + angular normalisation
//   EQLL   34649, EQSS 35928, RNORM1 37750   spinor E-coefficients
//   ERIFAST 12269-13132  first/second contraction, 16 m-sign combinations
//   CLMMTG 13841 / CLMMTZ 13135  J/K digestion (batch types 1 and 5)
//   CLMFAST 11489-12266  loop structure, selection rules, stage gating
//   EQLS 34937, EQSL 35433  sigma-coupled LS/SL E-coefficients
//   BRTFAST 17060, BIIFAST 18337, BRTMTG 19815 / BRTMTZ 19172  Breit exchange
//   ONEEL 6996, OVRLP 6683  overlap, nuclear attraction, kinetic coupling
//   FOCKIND 2582, CARTIND 2651  index layouts

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <deque>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef std::complex<double> cplx;

namespace {

const double PI = 3.1415926535897932;
const double PI12 = 1.7724538509055160;
const double PI52 = 1.7493418327624863e1;

constexpr int ntuv(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }

// ---------------------------------------------------------------------------
// Hermite index order (CARTIND, bertha-scf.f:2651-2703): lambda ascending,
// then t ascending, then u ascending, v = lambda - t - u.
// ---------------------------------------------------------------------------
const int MAXL = 24;
struct Cart {
  int idx[MAXL + 1][MAXL + 1][MAXL + 1];
  int t[ntuv(MAXL) + 1], u[ntuv(MAXL) + 1], v[ntuv(MAXL) + 1],
      lam[ntuv(MAXL) + 1];
  Cart() {
    int n = 0;
    for (int L = 0; L <= MAXL; ++L)
      for (int a = 0; a <= L; ++a)
        for (int b = 0; b <= L - a; ++b) {
          int c = L - a - b;
          idx[a][b][c] = n;
          t[n] = a; u[n] = b; v[n] = c; lam[n] = L;
          ++n;
        }
  }
};
const Cart &cart() {
  static Cart c;
  return c;
}

// ---------------------------------------------------------------------------
// Boys function F_m(T), m = 0..lam (FUNFM, bertha-scf.f:32465-32619, with
// the regime boundaries of RMAKE, bertha-scf.f:31927-31929).
// ---------------------------------------------------------------------------
void boys(double T, int lam, double *F) {
  const double EPSZR = 1.0e-11, EPSPL = 17.0, EPSAS = 30.0;
  const double A0 = 4.994501191201870e-1, B0 = 4.551838436668326e-1;
  if (T <= EPSZR) {
    for (int m = 0; m <= lam; ++m) F[m] = 1.0 / double(2 * m + 1);
  } else if (T <= EPSPL) {
    // 60-term power series at the top order, then downward recursion
    double txp = std::exp(-T), tt2 = 2.0 * T, term = 1.0, s = 1.0;
    for (int k = 1; k <= 60; ++k) {
      term = term * tt2 / double(2 * lam + 2 * k + 1);
      s += term;
    }
    F[lam] = s * txp / double(2 * lam + 1);
    for (int m = lam - 1; m >= 0; --m)
      F[m] = (tt2 * F[m + 1] + txp) / double(2 * m + 1);
  } else if (T <= EPSAS) {
    // rational seed times exp(-T), then upward recursion
    double txp = std::exp(-T), tt2 = 2.0 * T;
    F[0] = 0.5 * PI12 / std::sqrt(T) - txp * (A0 / (B0 + T));
    for (int m = 0; m < lam; ++m)
      F[m + 1] = (double(2 * m + 1) * F[m] - txp) / tt2;
  } else {
    // asymptotic, exp(-T) dropped
    double tt2 = 2.0 * T;
    F[0] = 0.5 * PI12 / std::sqrt(T);
    for (int m = 0; m < lam; ++m) F[m + 1] = double(2 * m + 1) * F[m] / tt2;
  }
}

// ---------------------------------------------------------------------------
// R-integrals R_{tuv}(alpha, P-Q), t+u+v <= lam (RMAKE, bertha-scf.f:31900).
// qp = Q - P as in ERIFAST (bertha-scf.f:12585-12587); the recursion uses
// P - Q = -qp.  Output indexed in CARTIND order.
// ---------------------------------------------------------------------------
void rints(const double qp[3], double alpha, int lam, double *R) {
  const Cart &C = cart();
  double T = alpha * (qp[0] * qp[0] + qp[1] * qp[1] + qp[2] * qp[2]);
  double F[MAXL + 2];
  boys(T, lam, F);
  double X = -qp[0], Y = -qp[1], Z = -qp[2];
  int nt = ntuv(lam);
  std::vector<double> cur(nt, 0.0), nxt(nt, 0.0);
  // level n = lam .. 0 ; at level n entries with t+u+v <= lam-n are valid
  double m2a = -2.0 * alpha;
  for (int n = lam; n >= 0; --n) {
    int top = lam - n;
    nxt[0] = std::pow(m2a, n) * F[n];
    for (int k = 1; k < ntuv(top); ++k) {
      int t = C.t[k], u = C.u[k], v = C.v[k];
      double val;
      if (t > 0) {
        val = X * cur[C.idx[t - 1][u][v]];
        if (t > 1) val += double(t - 1) * cur[C.idx[t - 2][u][v]];
      } else if (u > 0) {
        val = Y * cur[C.idx[t][u - 1][v]];
        if (u > 1) val += double(u - 1) * cur[C.idx[t][u - 2][v]];
      } else {
        val = Z * cur[C.idx[t][u][v - 1]];
        if (v > 1) val += double(v - 1) * cur[C.idx[t][u][v - 2]];
      }
      nxt[k] = val;
    }
    std::swap(cur, nxt);
  }
  for (int k = 0; k < nt; ++k) R[k] = cur[k];
}

// ---------------------------------------------------------------------------
// Hermite expansions of products of solid harmonic Gaussians (Saunders
// recursion, EVRS/ESTEPLM/ESTEPL/ESTEPN, bertha-scf.f:36981-37747).
// A vector holds coefficients E_{tuv} of Lambda_{tuv}(r; p, P) up to a degree.
// ---------------------------------------------------------------------------
struct PairGeom {
  double p, PA[3], PB[3], PA2, PB2, rkab;
};

PairGeom pair_geom(double ea, const double *A, double eb, const double *B) {
  PairGeom g;
  g.p = ea + eb;
  double ab2 = 0.0;
  for (int x = 0; x < 3; ++x) {
    double P = (ea * A[x] + eb * B[x]) / g.p;
    g.PA[x] = P - A[x];
    g.PB[x] = P - B[x];
    ab2 += (A[x] - B[x]) * (A[x] - B[x]);
  }
  g.PA2 = g.PA[0] * g.PA[0] + g.PA[1] * g.PA[1] + g.PA[2] * g.PA[2];
  g.PB2 = g.PB[0] * g.PB[0] + g.PB[1] * g.PB[1] + g.PB[2] * g.PB[2];
  g.rkab = std::exp(-(ea * eb * ab2) / g.p);
  return g;
}

typedef std::vector<cplx> HVec;

// out (degree L+1) += f * (x_c + i*phm*y_c) * in (degree L)   [sectoral]
//   or         += f * z_c * in                               [axial]
// using x_c Lambda_t = X Lambda_t + Lambda_{t+1}/(2p) + t Lambda_{t-1}
void mul_linear(const HVec &in, int L, HVec &out, double f, bool axial,
                double phm, const double *PC, double p) {
  const Cart &C = cart();
  const cplx I(0.0, 1.0);
  double inv2p = f / (2.0 * p);
  for (int k = 0; k < ntuv(L); ++k) {
    cplx e = in[k];
    if (e == cplx(0.0)) continue;
    int t = C.t[k], u = C.u[k], v = C.v[k];
    if (axial) {
      out[k] += f * PC[2] * e;
      out[C.idx[t][u][v + 1]] += inv2p * e;
      if (v > 0) out[C.idx[t][u][v - 1]] += f * double(v) * e;
    } else {
      cplx iy = phm * I;
      out[k] += f * PC[0] * e + iy * (f * PC[1]) * e;
      out[C.idx[t + 1][u][v]] += inv2p * e;
      out[C.idx[t][u + 1][v]] += iy * inv2p * e;
      if (t > 0) out[C.idx[t - 1][u][v]] += f * double(t) * e;
      if (u > 0) out[C.idx[t][u - 1][v]] += iy * (f * double(u)) * e;
    }
  }
}

// out (degree L+2) += f * r_c^2 * in (degree L)
void mul_r2(const HVec &in, int L, HVec &out, double f, const double *PC,
            double PC2, double p) {
  const Cart &C = cart();
  double p2 = 2.0 * p, p22 = p2 * p2;
  for (int k = 0; k < ntuv(L); ++k) {
    cplx e = in[k];
    if (e == cplx(0.0)) continue;
    int t = C.t[k], u = C.u[k], v = C.v[k];
    double tt = PC2 + double(2 * (t + u + v) + 3) / p2;
    out[k] += f * tt * e;
    out[C.idx[t + 2][u][v]] += (f / p22) * e;
    out[C.idx[t][u + 2][v]] += (f / p22) * e;
    out[C.idx[t][u][v + 2]] += (f / p22) * e;
    out[C.idx[t + 1][u][v]] += (f * PC[0] / p) * e;
    out[C.idx[t][u + 1][v]] += (f * PC[1] / p) * e;
    out[C.idx[t][u][v + 1]] += (f * PC[2] / p) * e;
    if (t > 0) out[C.idx[t - 1][u][v]] += (f * 2.0 * t * PC[0]) * e;
    if (u > 0) out[C.idx[t][u - 1][v]] += (f * 2.0 * u * PC[1]) * e;
    if (v > 0) out[C.idx[t][u][v - 1]] += (f * 2.0 * v * PC[2]) * e;
    if (t > 1) out[C.idx[t - 2][u][v]] += (f * double(t * (t - 1))) * e;
    if (u > 1) out[C.idx[t][u - 2][v]] += (f * double(u * (u - 1))) * e;
    if (v > 1) out[C.idx[t][u][v - 2]] += (f * double(v * (v - 1))) * e;
  }
}

// Multiply the expansion `cur` (degree L) by the unnormalised Schiff-phase
// solid harmonic S_{l,m} about centre c (ESTEPLM then ESTEPL).  Returns the
// new degree.
int apply_solid(HVec &cur, int L, int l, int m, const double *PC, double PC2,
                double p) {
  int am = std::abs(m);
  int NT = ntuv(MAXL);
  double phm = (m >= 0) ? 1.0 : -1.0;
  // sectoral steps: S_{k+1,+-(k+1)} = (2k+1)(x +- i y) S_{k,+-k}   Eq.(64)
  for (int k = 0; k < am; ++k) {
    HVec nx(NT, cplx(0.0));
    mul_linear(cur, L, nx, double(2 * k + 1), false, phm, PC, p);
    cur.swap(nx);
    ++L;
  }
  if (l <= am) return L;
  // first axial step: S_{|m|+1,m} = (2|m|+1) z S_{|m|,m}
  HVec prev = cur;
  {
    HVec nx(NT, cplx(0.0));
    mul_linear(cur, L, nx, double(2 * am + 1), true, 0.0, PC, p);
    cur.swap(nx);
    ++L;
  }
  // three-term steps for l = |m|+1 .. l-1
  for (int ls = am + 1; ls <= l - 1; ++ls) {
    double rlm1 = double(2 * ls + 1) / double(ls - am + 1);
    double rlm2 = -double(ls + am) / double(ls - am + 1);
    HVec nx(NT, cplx(0.0));
    mul_linear(cur, L, nx, rlm1, true, 0.0, PC, p);
    mul_r2(prev, L - 1, nx, rlm2, PC, PC2, p);
    prev.swap(cur);
    cur.swap(nx);
    ++L;
  }
  return L;
}

double rfact(int n) {
  double r = 1.0;
  for (int i = 2; i <= n; ++i) r *= double(i);
  return r;
}

// ESGTF (bertha-scf.f:36900): coefficients of Y*_{l1,m1}(r_A) Y_{l2,m2}(r_B)
// (Condon-Shortley, times the radial powers r_A^l1 r_B^l2) in the Hermite
// basis, with the extra factors (r_A^2)^na (r_B^2)^nb of ESTEPN.  The output
// has degree l1+l2+2(na+nb).  Zero when |m|>l.
HVec esgtf(int l1, int m1, int l2, int m2, int na, int nb, const PairGeom &g) {
  int NT = ntuv(MAXL);
  HVec cur(NT, cplx(0.0));
  if (std::abs(m1) > l1 || std::abs(m2) > l2) return cur;
  cur[0] = g.rkab;
  int L = 0;
  L = apply_solid(cur, L, l1, -m1, g.PA, g.PA2, g.p);
  L = apply_solid(cur, L, l2, m2, g.PB, g.PB2, g.p);
  double phs1 = (m1 > 0 && (m1 % 2)) ? -1.0 : 1.0;
  double phs2 = (m2 > 0 && (m2 % 2)) ? -1.0 : 1.0;
  double dgl = double((2 * l1 + 1) * (2 * l2 + 1));
  double cg1 = rfact(l1 - std::abs(m1)) / rfact(l1 + std::abs(m1));
  double cg2 = rfact(l2 - std::abs(m2)) / rfact(l2 + std::abs(m2));
  double ang = phs1 * phs2 * (0.25 / PI) * std::sqrt(dgl * cg1 * cg2);
  for (int k = 0; k < ntuv(L); ++k) cur[k] *= ang;
  // radial r^2 factors are applied after normalisation, as in EQSS
  for (int s = 0; s < na; ++s) {
    HVec nx(NT, cplx(0.0));
    mul_r2(cur, L, nx, 1.0, g.PA, g.PA2, g.p);
    cur.swap(nx);
    L += 2;
  }
  for (int s = 0; s < nb; ++s) {
    HVec nx(NT, cplx(0.0));
    mul_r2(cur, L, nx, 1.0, g.PB, g.PB2, g.p);
    cur.swap(nx);
    L += 2;
  }
  return cur;
}

inline int lval(int kqn) { return kqn < 0 ? -kqn - 1 : kqn; }

// Radial normalisation (RNORM1, bertha-scf.f:37750): large (L) and
// kinetically balanced small (S) components.
double rnorm(double ex, int l, bool small) {
  if (!small)
    return std::exp(0.5 * (std::log(2.0) - std::lgamma(l + 1.5) +
                           (l + 1.5) * std::log(2.0 * ex)));
  return std::exp(0.5 * (std::log(2.0) - std::lgamma(l + 2.5) +
                         (l + 0.5) * std::log(2.0 * ex)));
}

// Clebsch-Gordan coefficients of a 2-spinor: upper and lower components.
// kqn, jqn = 2j, mqn = 2m (signed).  For the small component the -kappa
// formula applies (EQLL bertha-scf.f:34712-34727 / EQSS 35990-36005).
void cg_pair(int kqn, int mqn, bool small, double &cu, double &cl) {
  int jqn = 2 * std::abs(kqn) - 1;
  bool neg = (kqn < 0);
  if (small) neg = !neg;
  if (neg) {
    cu = std::sqrt(double(jqn + mqn) / double(2 * jqn));
    cl = std::sqrt(double(jqn - mqn) / double(2 * jqn));
  } else {
    cu = -std::sqrt(double(jqn - mqn + 2) / double(2 * jqn + 4));
    cl = std::sqrt(double(jqn + mqn + 2) / double(2 * jqn + 4));
  }
}

// Radial terms of one component of a G-spinor as (coefficient, power of
// r^2) multiplying r^l' Y_l': large: (1,0); kinetically balanced small:
// kappa<0 -> (-2a,0) with l'=l+1; kappa>0 -> (2l+1,0), (-2a,1) with l'=l-1
// (EQSS bertha-scf.f:36010-36029, EQLS :34990-35000).
struct RTerm { double c; int n; };
int radial_terms(int kq, double ex, bool small, RTerm *t, int &lp) {
  int l = lval(kq);
  if (!small) { lp = l; t[0] = {1.0, 0}; return 1; }
  if (kq < 0) { lp = l + 1; t[0] = {-2.0 * ex, 0}; return 1; }
  lp = l - 1;
  t[0] = {double(2 * l + 1), 0};
  t[1] = {-2.0 * ex, 1};
  return 2;
}

// Spinor overlap E-coefficients psi_a^+ sigma_q psi_b for one primitive pair
// (EQLL :34649, EQSS :35928, EQLS :34937, EQSL :35433): components small_a,
// small_b; iq = 0 (unit), 1 (sigma_x), 2 (sigma_y), 3 (sigma_z).  mqa, mqb
// are signed 2m.  The small component carries the factor i of the
// reference (LS x i, SL x -i).  Degree l'_a + l'_b + 2(n_a + n_b).
HVec eq_pair_q(int ka, int mqa, double ea, const double *A, int kb, int mqb, double eb,
               const double *B, bool sa, bool sb, int iq) {
  const double SENS = 1.0e-14;
  PairGeom g = pair_geom(ea, A, eb, B);
  int la = lval(ka), lb = lval(kb);
  int NT = ntuv(MAXL);
  HVec E(NT, cplx(0.0));
  double cau, cal, cbu, cbl;
  cg_pair(ka, mqa, sa, cau, cal);
  cg_pair(kb, mqb, sb, cbu, cbl);
  RTerm ta[2], tb[2];
  int l1, l2;
  int na = radial_terms(ka, ea, sa, ta, l1), nb = radial_terms(kb, eb, sb, tb, l2);
  // spin products: (A spin, B spin, weight) per Pauli matrix
  struct SpinTerm { int ua, ub; double w; };
  SpinTerm st[2];
  if (iq == 0) { st[0] = {0, 0, 1.0}; st[1] = {1, 1, 1.0}; }
  else if (iq == 3) { st[0] = {0, 0, 1.0}; st[1] = {1, 1, -1.0}; }
  else if (iq == 1) { st[0] = {0, 1, 1.0}; st[1] = {1, 0, 1.0}; }
  else { st[0] = {0, 1, -1.0}; st[1] = {1, 0, 1.0}; }
  int deg = 0;
  for (int s = 0; s < 2; ++s) {
    double cab = (st[s].ua == 0 ? cau : cal) * (st[s].ub == 0 ? cbu : cbl);
    if (std::fabs(cab) < SENS) continue;
    int m1 = st[s].ua == 0 ? (mqa - 1) / 2 : (mqa + 1) / 2;
    int m2 = st[s].ub == 0 ? (mqb - 1) / 2 : (mqb + 1) / 2;
    for (int i = 0; i < na; ++i)
      for (int j = 0; j < nb; ++j) {
        HVec es = esgtf(l1, m1, l2, m2, ta[i].n, tb[j].n, g);
        int d = l1 + l2 + 2 * (ta[i].n + tb[j].n);
        deg = std::max(deg, d);
        double c = st[s].w * cab * ta[i].c * tb[j].c;
        for (int k = 0; k < ntuv(d); ++k) E[k] += c * es[k];
      }
  }
  double nrm = rnorm(ea, la, sa) * rnorm(eb, lb, sb);
  cplx ph(1.0, 0.0);
  if (sa && !sb) ph = cplx(0.0, -1.0);
  if (!sa && sb) ph = cplx(0.0, 1.0);
  if (iq == 2) ph *= cplx(0.0, 1.0);
  int dmax = la + lb + (sa ? 1 : 0) + (sb ? 1 : 0);
  HVec out(E.begin(), E.begin() + ntuv(dmax));
  for (cplx &v : out) v *= nrm * ph;
  return out;
}

// LL / SS E-coefficients (the Coulomb densities)
HVec eq_pair(int ka, int mqa, double ea, const double *A, int kb, int mqb,
             double eb, const double *B, bool small) {
  return eq_pair_q(ka, mqa, ea, A, kb, mqb, eb, B, small, small, 0);
}

// ---------------------------------------------------------------------------
// Basis and Fock layout (CARDIN / FOCKIND, bertha-scf.f:150, 2582)
// ---------------------------------------------------------------------------
struct Basis {
  int ncnt;
  std::vector<double> xyz;            // [ncnt][3]
  std::vector<int> lmax;              // [ncnt]
  std::vector<std::vector<std::vector<double>>> ex;  // [cnt][l][ibas]
  // Fock offsets lrge[cnt][ka][mqn-1], ka = 0.., mqn index 0..(2*|kappa|)-1
  std::vector<std::vector<std::vector<int>>> lrge;
  int ndim, nskp;
};

inline int kappa_of(int ka) {  // KAPA(KA) with KA 1-based: 1->-1, 2l->l, 2l+1->-l-1
  if (ka == 1) return -1;
  return (ka % 2 == 0) ? ka / 2 : -(ka / 2) - 1;
}

void fock_layout(Basis &b, bool norl) {
  b.lrge.assign(b.ncnt, {});
  int ilst = 0;
  int total = 0;
  for (int iz = 0; iz < b.ncnt; ++iz) {
    int nkap = 2 * b.lmax[iz] + 1;
    b.lrge[iz].assign(nkap + 1, std::vector<int>(2 * 14 + 2, -1));
    for (int l = 0; l <= b.lmax[iz]; ++l)
      total += 4 * (2 * l + 1) * int(b.ex[iz][l].size());
  }
  for (int iz = 0; iz < b.ncnt; ++iz) {
    int nkap = 2 * b.lmax[iz] + 1;
    for (int imv = 0; imv <= 13; ++imv) {
      int mqn = 2 * imv + 1;
      for (int sgn = 0; sgn < 2; ++sgn)
        for (int ka = 1; ka <= nkap; ++ka) {
          int kq = kappa_of(ka);
          int nbas = int(b.ex[iz][lval(kq)].size());
          if (2 * std::abs(kq) - 1 >= mqn) {
            b.lrge[iz][ka][mqn - 1 + sgn] = ilst;
            ilst += nbas;
          }
        }
    }
  }
  b.ndim = norl ? total / 2 : total;
  b.nskp = norl ? 0 : total / 2;
}

int ncntrs(int a, int b, int c, int d) {
  int s[4] = {a, b, c, d};
  std::sort(s, s + 4);
  int n = 1;
  for (int i = 1; i < 4; ++i)
    if (s[i] != s[i - 1]) ++n;
  return n;
}

// Options of the Fock build (HFSCF toggles, bertha-scf.f:5215-5257)
struct Opts {
  int ilev;     // integral inclusion stage 1..4
  int isym;     // 0 general (CLMMTG), 1 linear, 2 atomic (CLMMTZ)
  int hmlt;     // 0 NORL, 1 BARE, 2 relativistic (DHFR/DHFP/DHFB/DHFQ)
  int racah1;   // skip one-centre quartets
  int ssssi3, ssssi4;
};

// ERIFAST second contraction result for one (ab,cd) label pair and one kl
// element: the 16 m-sign combinations, index 8*sa+4*sb+2*sc+sd (s=1 for +).
struct Eri16 { cplx v[16]; };

// The 16 combinations from G(ab) (first contraction, sets 11 and 21) and the
// cd E-coefficients, following ERIFAST bertha-scf.f:12809-13119.
void second_contraction(const cplx *g11, const cplx *g21, const cplx *e11cd,
                        const cplx *e21cd, int ncd, double pab, double pcd,
                        Eri16 &o) {
  const Cart &C = cart();
  cplx s1(0), s1c(0), s2(0), s2c(0), s3(0), s3c(0), s4(0), s4c(0);
  for (int k = 0; k < ncd; ++k) {
    double z = (C.lam[k] & 1) ? -1.0 : 1.0;
    cplx a = z * e11cd[k], b = z * e21cd[k];
    s1 += a * g11[k];
    s1c += a * std::conj(g11[k]);
    s2 += b * g11[k];
    s2c += b * std::conj(g11[k]);
    s3 += a * g21[k];
    s3c += a * std::conj(g21[k]);
    s4 += b * g21[k];
    s4c += b * std::conj(g21[k]);
  }
  double pabcd = pab * pcd;
  cplx *r = o.v;
  // set 1: (--|--)=0, (++|--)=12, (++|++)=15, (--|++)=3
  r[0] = s1;
  r[12] = pab * s1c;
  r[15] = pabcd * std::conj(r[0]);
  r[3] = pabcd * std::conj(r[12]);
  // set 2: (--|+-)=2, (++|+-)=14, (++|-+)=13, (--|-+)=1
  r[2] = s2;
  r[14] = pab * s2c;
  r[13] = -pabcd * std::conj(r[2]);
  r[1] = -pabcd * std::conj(r[14]);
  // set 3: (+-|--)=8, (-+|--)=4, (-+|++)=7, (+-|++)=11
  r[8] = s3;
  r[4] = -pab * s3c;
  r[7] = -pabcd * std::conj(r[8]);
  r[11] = -pabcd * std::conj(r[4]);
  // set 4: (+-|+-)=10, (-+|+-)=6, (-+|-+)=5, (+-|-+)=9
  r[10] = s4;
  r[6] = -pab * s4c;
  r[5] = pabcd * std::conj(r[10]);
  r[9] = pabcd * std::conj(r[6]);
}

struct Mat {
  cplx *p;
  int ld;
  cplx &operator()(int i, int j) const { return p[i + (size_t)ld * j]; }
};

// CLMMTG / CLMMTZ batch types 1 (direct) and 5 (exchange) for one kl element.
// na[s], nb[s], nc[s], nd[s]: Fock indices of the four spinors for m-sign s.
void digest(const Eri16 &rr, const int na[2], const int nb[2], const int nc[2],
            const int nd[2], const Mat &D, Mat &GD, Mat &GX, int isym) {
  if (isym == 0) {
    for (int sa = 0; sa < 2; ++sa)
      for (int sb = 0; sb < 2; ++sb)
        for (int sc = 0; sc < 2; ++sc)
          for (int sd = 0; sd < 2; ++sd) {
            cplx v = rr.v[8 * sa + 4 * sb + 2 * sc + sd];
            GD(na[sa], nb[sb]) += v * D(nc[sc], nd[sd]);
            GX(na[sa], nd[sd]) += v * D(nc[sc], nb[sb]);
          }
  } else {
    // real Fock matrix case: only equal-sign direct blocks (sa=sb, sc=sd)
    // and exchange blocks with sa=sd, sb=sc, real parts only
    for (int s = 0; s < 2; ++s)
      for (int t = 0; t < 2; ++t) {
        double vd = rr.v[8 * s + 4 * s + 2 * t + t].real();
        GD(na[s], nb[s]) += vd * D(nc[t], nd[t]).real();
        double vx = rr.v[8 * s + 4 * t + 2 * t + s].real();
        GX(na[s], nd[s]) += vx * D(nc[t], nb[t]).real();
      }
  }
}

// One spinor label (kappa index, |m| index) on a centre with its E data.
struct Label {
  int ka;   // KA, 1-based
  int kq;   // kappa
  int ma;   // |m| + 1/2, 1..|kappa|
};

std::vector<Label> labels_for(int l) {
  std::vector<Label> out;
  for (int n = (l == 0 ? 1 : 0); n <= 1; ++n) {
    int ka = 2 * l + n;
    int kq = kappa_of(ka);
    for (int ma = 1; ma <= std::abs(kq); ++ma) out.push_back({ka, kq, ma});
  }
  return out;
}

// E-coefficients of all labels of a (centre A, l_a; centre B, l_b) block for
// all primitive pairs, sets 11 (-|ma|,-|mb|) and 21 (+|ma|,-|mb|).
struct EBlock {
  int nlab_a, nlab_b, na, nb, nt;
  std::vector<Label> la, lb;
  std::vector<cplx> e;  // [lab_a][lab_b][set][ij][nt]
  const cplx *at(int ia, int ib, int set, int ij) const {
    return &e[((((size_t)ia * nlab_b + ib) * 2 + set) * (na * nb) + ij) * nt];
  }
};

EBlock make_eblock(const Basis &b, int ca, int lA, int cb, int lB, bool small) {
  EBlock E;
  E.la = labels_for(lA);
  E.lb = labels_for(lB);
  E.nlab_a = int(E.la.size());
  E.nlab_b = int(E.lb.size());
  const std::vector<double> &xa = b.ex[ca][lA], &xb = b.ex[cb][lB];
  E.na = int(xa.size());
  E.nb = int(xb.size());
  E.nt = ntuv(lA + lB + (small ? 2 : 0));
  E.e.assign((size_t)E.nlab_a * E.nlab_b * 2 * E.na * E.nb * E.nt, cplx(0));
  const double *A = &b.xyz[3 * ca], *B = &b.xyz[3 * cb];
  for (int ia = 0; ia < E.nlab_a; ++ia)
    for (int ib = 0; ib < E.nlab_b; ++ib)
      for (int set = 0; set < 2; ++set) {
        int mqa = (set == 0 ? -1 : 1) * (2 * E.la[ia].ma - 1);
        int mqb = -(2 * E.lb[ib].ma - 1);
        for (int i = 0; i < E.na; ++i)
          for (int j = 0; j < E.nb; ++j) {
            HVec h = eq_pair(E.la[ia].kq, mqa, xa[i], A, E.lb[ib].kq, mqb,
                             xb[j], B, small);
            cplx *dst = const_cast<cplx *>(E.at(ia, ib, set, i * E.nb + j));
            for (int k = 0; k < E.nt; ++k) dst[k] = h[k];
          }
      }
  return E;
}

inline double phase_pair(int kqa, int ma, int kqb, int mb) {
  // ISIGN(1,KA*KB)*(-1)**((MQNA-MQNB)/2), MQN = 2|m| (bertha-scf.f:12810)
  double s = ((kqa > 0) == (kqb > 0)) ? 1.0 : -1.0;
  int d = (2 * ma - 1 - (2 * mb - 1)) / 2;
  return (d % 2 == 0) ? s : -s;
}

// Selection rules of CLMFAST for one label quartet (bertha-scf.f:11914-11939
// and 11843-11890); with breit, those of BRTFAST (:17432-17486), whose
// tensor-order rule also keeps both parities odd with nu > 0 (the magnetic
// terms).  Returns false if the quartet is skipped.
bool label_rules(const Opts &o, int mcnt, const Label *lab, const int *lq, bool breit = false) {
  int mq[4], jq[4];
  for (int i = 0; i < 4; ++i) {
    mq[i] = 2 * lab[i].ma - 1;
    jq[i] = 2 * std::abs(lab[i].kq) - 1;
  }
  if (mcnt == 1 && !o.racah1) {
    int nui = std::max(std::abs(jq[0] - jq[1]) / 2, std::abs(jq[2] - jq[3]) / 2);
    int nuf = std::min((jq[0] + jq[1]) / 2, (jq[2] + jq[3]) / 2);
    if (nui > nuf) return false;
    bool selk = false;
    for (int nu = nui; nu <= nuf; ++nu) {
      int pab = (lq[0] + lq[1] + nu) % 2, pcd = (lq[2] + lq[3] + nu) % 2;
      if ((pab == 0 && pcd == 0) || (breit && pab == 1 && pcd == 1 && nu != 0)) selk = true;
    }
    if (!selk) return false;
  }
  if (o.isym == 1 || o.isym == 2) {
    bool ok = (mq[0] == mq[1] && mq[2] == mq[3]) ||
              (mq[0] == mq[2] && mq[1] == mq[3]) ||
              (mq[0] == mq[3] && mq[1] == mq[2]);
    if (!ok) return false;
  }
  if (mcnt == 1 && !o.racah1) {
    bool selm = false;
    for (int a = 0; a < 2; ++a)
      for (int bb = 0; bb < 2; ++bb)
        for (int c = 0; c < 2; ++c)
          for (int d = 0; d < 2; ++d) {
            int ja = mq[0] * (a ? 1 : -1), jb = mq[1] * (bb ? 1 : -1);
            int jc = mq[2] * (c ? 1 : -1), jd = mq[3] * (d ? 1 : -1);
            if (ja - jb == jd - jc) selm = true;
          }
    if (!selm) return false;
  }
  return true;
}

// Stage gating (bertha-scf.f:12045-12084).  itt: 1 LL|LL, 2 LL|SS,
// 3 SS|LL, 4 SS|SS.
bool stage_ok(const Opts &o, int mcnt, int itt) {
  if (o.ilev == 1 && itt > 1 && mcnt != 1) return false;
  if (o.ilev == 2 && itt > 3 && mcnt != 1) return false;
  if (o.ilev == 3 && itt == 4) {
    if (o.ssssi3 && mcnt == 3) return false;
    if (o.ssssi4 && mcnt == 4) return false;
  }
  return true;
}

// Multi-centre Coulomb Fock build with the reference's INTSYM = .FALSE.
// semantics: every ordered quartet, batch types 1 and 5 only.
void fock_full(const Basis &b, const Opts &o, const Mat &D, Mat &GD, Mat &GX) {
  // E-coefficient blocks are generated once per (centre, l) pair and
  // component type, as EQSAVE does before the SCF (bertha-scf.f:5287)
  std::deque<EBlock> ecache;  // deque: references stay valid on growth
  std::vector<int> ekey;
  auto eblock = [&](int c1, int l1, int c2, int l2, int sm) -> const EBlock & {
    int key = (((c1 * 16 + l1) * 1024 + c2) * 16 + l2) * 2 + sm;
    for (size_t i = 0; i < ekey.size(); ++i)
      if (ekey[i] == key) return ecache[i];
    ekey.push_back(key);
    ecache.push_back(make_eblock(b, c1, l1, c2, l2, sm != 0));
    return ecache.back();
  };
  for (int j = 0; j < b.ndim; ++j)
    for (int i = 0; i < b.ndim; ++i) GD(i, j) = GX(i, j) = 0.0;
  if (o.hmlt == 1) return;
  std::vector<int> tcomp;
  if (o.hmlt == 0) tcomp = {0};
  else tcomp = {1, 0};  // SS then LL, as ITSTRT=4, ITSKIP=-3
  const Cart &C = cart();
  // OpenMP inside each class: every thread digests into its own matrices,
  // summed in thread order at the end (the serial result up to rounding)
  int nthr = 1;
#ifdef _OPENMP
  nthr = omp_get_max_threads();
#endif
  const size_t nn = (size_t)b.ndim * b.ndim;
  std::vector<std::vector<cplx>> accd(nthr), accx(nthr);
  for (int ca = 0; ca < b.ncnt; ++ca)
  for (int cb = 0; cb < b.ncnt; ++cb)
  for (int cc = 0; cc < b.ncnt; ++cc)
  for (int cd = 0; cd < b.ncnt; ++cd) {
    int mcnt = ncntrs(ca, cb, cc, cd);
    if (mcnt == 1 && o.racah1) continue;
    for (int lA = 0; lA <= b.lmax[ca]; ++lA)
    for (int lB = 0; lB <= b.lmax[cb]; ++lB)
    for (int lC = 0; lC <= b.lmax[cc]; ++lC)
    for (int lD = 0; lD <= b.lmax[cd]; ++lD) {
      if (mcnt == 1 && !o.racah1 && ((lA + lB) % 2) != ((lC + lD) % 2))
        continue;
      int lq[4] = {lA, lB, lC, lD};
      for (int t1 : tcomp)
      for (int t2 : tcomp) {
        int itt = 1 + 2 * t1 + t2;
        if (!stage_ok(o, mcnt, itt)) continue;
        const EBlock &Eab = eblock(ca, lA, cb, lB, t1);
        const EBlock &Ecd = eblock(cc, lC, cd, lD, t2);
        int nab = Eab.nt, ncd = Ecd.nt;
        int lam = (lA + lB + 2 * t1) + (lC + lD + 2 * t2);
        int nij = Eab.na * Eab.nb, nkl = Ecd.na * Ecd.nb;
        // R-integral batch PRE*R for all (ij,kl)
        std::vector<double> R((size_t)nij * nkl * ntuv(lam));
        const double *A = &b.xyz[3 * ca], *B = &b.xyz[3 * cb];
        const double *Cc = &b.xyz[3 * cc], *Dd = &b.xyz[3 * cd];
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic)
#endif
        for (int ijr = 0; ijr < nij; ++ijr) {
          int i = ijr / Eab.nb, j = ijr % Eab.nb;
          double ei = b.ex[ca][lA][i], ej = b.ex[cb][lB][j], eij = ei + ej;
          double P[3];
          for (int x = 0; x < 3; ++x) P[x] = (A[x] * ei + B[x] * ej) / eij;
          for (int k = 0; k < Ecd.na; ++k)
          for (int l = 0; l < Ecd.nb; ++l) {
            double ek = b.ex[cc][lC][k], el = b.ex[cd][lD][l], ekl = ek + el;
            double qp[3];
            for (int x = 0; x < 3; ++x)
              qp[x] = (Cc[x] * ek + Dd[x] * el) / ekl - P[x];
            double aph = eij * ekl / (eij + ekl);
            double pre = 2.0 * PI52 / (std::sqrt(eij + ekl) * eij * ekl);
            double *r = &R[((size_t)(i * Eab.nb + j) * nkl + k * Ecd.nb + l) *
                           ntuv(lam)];
            rints(qp, aph, lam, r);
            for (int n = 0; n < ntuv(lam); ++n) r[n] *= pre;
          }
        }
        int offab = t1 ? b.nskp : 0, offcd = t2 ? b.nskp : 0;
        const long long nwork = (long long)Eab.nlab_a * Eab.nlab_b * nij;
#ifdef _OPENMP
#pragma omp parallel
#endif
        {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        if (accd[tid].empty()) {
          accd[tid].assign(nn, cplx(0));
          accx[tid].assign(nn, cplx(0));
        }
        Mat TD{accd[tid].data(), b.ndim}, TX{accx[tid].data(), b.ndim};
        std::vector<cplx> g11((size_t)nkl * ncd), g21((size_t)nkl * ncd);
#ifdef _OPENMP
#pragma omp for schedule(dynamic)
#endif
        for (long long w = 0; w < nwork; ++w) {
          int ij = (int)(w % nij), iab = (int)(w / nij);
          int ia = iab / Eab.nlab_b, ib = iab % Eab.nlab_b;
          int i = ij / Eab.nb, j = ij % Eab.nb;
          const Label &LA = Eab.la[ia], &LB = Eab.lb[ib];
          {
            const cplx *e11 = Eab.at(ia, ib, 0, ij), *e21 = Eab.at(ia, ib, 1, ij);
            // first contraction G(kl, t'u'v') for all kl
            for (int kl = 0; kl < nkl; ++kl) {
              const double *r = &R[((size_t)ij * nkl + kl) * ntuv(lam)];
              for (int q = 0; q < ncd; ++q) {
                cplx a(0), bq(0);
                for (int s = 0; s < nab; ++s) {
                  double rv = r[C.idx[C.t[s] + C.t[q]][C.u[s] + C.u[q]]
                                    [C.v[s] + C.v[q]]];
                  a += e11[s] * rv;
                  bq += e21[s] * rv;
                }
                g11[(size_t)kl * ncd + q] = a;
                g21[(size_t)kl * ncd + q] = bq;
              }
            }
            for (int ic = 0; ic < Ecd.nlab_a; ++ic)
            for (int id = 0; id < Ecd.nlab_b; ++id) {
              const Label &LC = Ecd.la[ic], &LD = Ecd.lb[id];
              Label quad[4] = {LA, LB, LC, LD};
              if (!label_rules(o, mcnt, quad, lq)) continue;
              double pab = phase_pair(LA.kq, LA.ma, LB.kq, LB.ma);
              double pcd = phase_pair(LC.kq, LC.ma, LD.kq, LD.ma);
              int na[2] = {b.lrge[ca][LA.ka][2 * LA.ma - 2] + offab + i,
                           b.lrge[ca][LA.ka][2 * LA.ma - 1] + offab + i};
              int nb[2] = {b.lrge[cb][LB.ka][2 * LB.ma - 2] + offab + j,
                           b.lrge[cb][LB.ka][2 * LB.ma - 1] + offab + j};
              for (int k = 0; k < Ecd.na; ++k)
              for (int l = 0; l < Ecd.nb; ++l) {
                int kl = k * Ecd.nb + l;
                Eri16 rr;
                second_contraction(&g11[(size_t)kl * ncd], &g21[(size_t)kl * ncd],
                                   Ecd.at(ic, id, 0, kl), Ecd.at(ic, id, 1, kl),
                                   ncd, pab, pcd, rr);
                int nc[2] = {b.lrge[cc][LC.ka][2 * LC.ma - 2] + offcd + k,
                             b.lrge[cc][LC.ka][2 * LC.ma - 1] + offcd + k};
                int nd[2] = {b.lrge[cd][LD.ka][2 * LD.ma - 2] + offcd + l,
                             b.lrge[cd][LD.ka][2 * LD.ma - 1] + offcd + l};
                digest(rr, na, nb, nc, nd, D, TD, TX, o.isym);
              }
            }
          }
        }
        }  // omp parallel
      }
    }
  }
  for (int t = 0; t < nthr; ++t) {
    if (accd[t].empty()) continue;
    for (int j = 0; j < b.ndim; ++j)
      for (int i = 0; i < b.ndim; ++i) {
        GD(i, j) += accd[t][i + (size_t)b.ndim * j];
        GX(i, j) += accx[t][i + (size_t)b.ndim * j];
      }
  }
}

// ---------------------------------------------------------------------------
// Breit / Gaunt interaction (BRTFAST :17060, BIIFAST :18337, BRTMTG :19815,
// BRTMTZ :19172)
// ---------------------------------------------------------------------------

// Spinor overlap E-coefficients with sigma_x, sigma_y, sigma_z of all labels
// of a (centre A, l_a; centre B, l_b) block, one component pair: LS (a large,
// b small, EQLS x i) or SL (a small, b large, EQSL x -i).  Degree
// l_a + l_b + 1.  Layout [lab_a][lab_b][set][q][ij][nt] (EILSGN :33644 keeps
// the same 2 sets x 3 Cartesian components per pair).
struct EBlockQ {
  int nlab_a, nlab_b, na, nb, nt;
  std::vector<Label> la, lb;
  std::vector<cplx> e;
  const cplx *at(int ia, int ib, int set, int q, int ij) const {
    return &e[(((((size_t)ia * nlab_b + ib) * 2 + set) * 3 + q) * (na * nb) + ij) * nt];
  }
};

EBlockQ make_eblock_q(const Basis &b, int ca, int lA, int cb, int lB, bool a_small) {
  EBlockQ E;
  E.la = labels_for(lA);
  E.lb = labels_for(lB);
  E.nlab_a = int(E.la.size());
  E.nlab_b = int(E.lb.size());
  const std::vector<double> &xa = b.ex[ca][lA], &xb = b.ex[cb][lB];
  E.na = int(xa.size());
  E.nb = int(xb.size());
  E.nt = ntuv(lA + lB + 1);
  E.e.assign((size_t)E.nlab_a * E.nlab_b * 2 * 3 * E.na * E.nb * E.nt, cplx(0));
  const double *A = &b.xyz[3 * ca], *B = &b.xyz[3 * cb];
  for (int ia = 0; ia < E.nlab_a; ++ia)
    for (int ib = 0; ib < E.nlab_b; ++ib)
      for (int set = 0; set < 2; ++set)
        for (int q = 0; q < 3; ++q) {
          int mqa = (set == 0 ? -1 : 1) * (2 * E.la[ia].ma - 1);
          int mqb = -(2 * E.lb[ib].ma - 1);
          for (int i = 0; i < E.na; ++i)
            for (int j = 0; j < E.nb; ++j) {
              HVec h = eq_pair_q(E.la[ia].kq, mqa, xa[i], A, E.lb[ib].kq, mqb, xb[j], B,
                                 a_small, !a_small, q + 1);
              cplx *dst = const_cast<cplx *>(E.at(ia, ib, set, q, i * E.nb + j));
              for (int k = 0; k < E.nt; ++k) dst[k] = h[k];
            }
        }
  return E;
}

// Breit kernel between Cartesian components i (electron 2, cd) and j
// (electron 1, ab) at Hermite index N = (t,u,v), from PRE*R-integrals of
// order |N|+2 (BIIFAST first contraction :18655-18880):
//   W_ij(N) = BFAC * (delta_ij R_N - T_ij(N)),
//   T_ij(N) = R_{N+e_i+e_j}/(2 alpha) - R_{N+e_i} PQ_j + N_j R_{N+e_i-e_j},
// PQ = Q - P, BFAC = -1/2.  Gaunt only: W_ij = -delta_ij R_N.
void breit_kernel(const double *R, const double *pq, double aph, int t, int u, int v,
                  bool gaunt, double W[3][3]) {
  const Cart &C = cart();
  int N[3] = {t, u, v};
  double rn = R[C.idx[t][u][v]];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      if (gaunt) {
        W[i][j] = i == j ? -rn : 0.0;
        continue;
      }
      int a[3] = {N[0], N[1], N[2]};
      a[i] += 1;
      a[j] += 1;
      double t1 = R[C.idx[a[0]][a[1]][a[2]]] * 0.5 / aph;
      a[j] -= 1;
      double t2 = R[C.idx[a[0]][a[1]][a[2]]] * pq[j];
      double t3 = 0.0;
      a[j] -= 1;
      if (a[j] >= 0) t3 = R[C.idx[a[0]][a[1]][a[2]]] * double(N[j]);
      W[i][j] = -0.5 * ((i == j ? rn : 0.0) - (t1 - t2 + t3));
    }
}

// BIIFAST for one primitive quartet and one ab label pair: the first
// contraction G_i(cd tuv), i = x, y, z, for sets 11 and 21.
// g11/g21: [3][ncd].  Wt: [ntuv(degab+degcd)][3][3] kernel table.
void bii_first(const EBlockQ &Eab, int ia, int ib, int ij, const std::vector<double> &Wt,
               int ncd, cplx *g11, cplx *g21) {
  const Cart &C = cart();
  int nab = Eab.nt;
  for (int i = 0; i < 3; ++i)
    for (int q = 0; q < ncd; ++q) {
      cplx x(0), y(0);
      for (int j = 0; j < 3; ++j) {
        const cplx *e11 = Eab.at(ia, ib, 0, j, ij), *e21 = Eab.at(ia, ib, 1, j, ij);
        for (int s = 0; s < nab; ++s) {
          int n = C.idx[C.t[s] + C.t[q]][C.u[s] + C.u[q]][C.v[s] + C.v[q]];
          double w = Wt[(size_t)n * 9 + 3 * i + j];
          x += e11[s] * w;
          y += e21[s] * w;
        }
      }
      g11[i * ncd + q] = x;
      g21[i * ncd + q] = y;
    }
}

// Breit phase of a pair: the Coulomb one negated (BRTFAST :17528-17533, BIIFAST :18899).
inline double phase_breit(int kqa, int ma, int kqb, int mb) {
  return -phase_pair(kqa, ma, kqb, mb);
}

// Second contraction summed over the Cartesian component (BIIFAST :18887-19145).
void bii_second(const cplx *g11, const cplx *g21, const EBlockQ &Ecd, int ic, int id,
                int kl, int ncd, double pab, double pcd, Eri16 &rr) {
  for (int s = 0; s < 16; ++s) rr.v[s] = 0.0;
  for (int i = 0; i < 3; ++i) {
    Eri16 part;
    second_contraction(g11 + i * ncd, g21 + i * ncd, Ecd.at(ic, id, 0, i, kl),
                       Ecd.at(ic, id, 1, i, kl), ncd, pab, pcd, part);
    for (int s = 0; s < 16; ++s) rr.v[s] += part.v[s];
  }
}

// Kernel table for one primitive quartet: PRE*R to order degab+degcd+2, then
// W for every N up to degab+degcd.
void bii_table(const double *P, double eij, const double *Q, double ekl, int degab,
               int degcd, bool gaunt, std::vector<double> &Wt) {
  int lamn = degab + degcd, lam = lamn + (gaunt ? 0 : 2);
  double qp[3];
  for (int x = 0; x < 3; ++x) qp[x] = Q[x] - P[x];
  double aph = eij * ekl / (eij + ekl);
  double pre = 2.0 * PI52 / (std::sqrt(eij + ekl) * eij * ekl);
  std::vector<double> R(ntuv(lam));
  rints(qp, aph, lam, R.data());
  for (double &r : R) r *= pre;
  const Cart &C = cart();
  Wt.assign((size_t)ntuv(lamn) * 9, 0.0);
  for (int n = 0; n < ntuv(lamn); ++n) {
    double W[3][3];
    breit_kernel(R.data(), qp, aph, C.t[n], C.u[n], C.v[n], gaunt, W);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) Wt[(size_t)n * 9 + 3 * i + j] = W[i][j];
  }
}

// BRTMTG / BRTMTZ batch type 5 (exchange) for one kl element.
void digest_x(const Eri16 &rr, const int na[2], const int nb[2], const int nc[2],
              const int nd[2], const Mat &D, Mat &BX, int isym) {
  if (isym == 0) {
    for (int sa = 0; sa < 2; ++sa)
      for (int sb = 0; sb < 2; ++sb)
        for (int sc = 0; sc < 2; ++sc)
          for (int sd = 0; sd < 2; ++sd)
            BX(na[sa], nd[sd]) += rr.v[8 * sa + 4 * sb + 2 * sc + sd] * D(nc[sc], nb[sb]);
  } else {
    for (int s = 0; s < 2; ++s)
      for (int t = 0; t < 2; ++t)
        BX(na[s], nd[s]) += rr.v[8 * s + 4 * t + 2 * t + s].real() * D(nc[t], nb[t]).real();
  }
}

// Closed-shell multi-centre Breit exchange matrix BXCH (BRTFAST with the
// direct matrix zero, NOPN = 0).  The reference evaluates only (LS|LS)
// batches and reaches the other component classes through integral
// permutation symmetry; this restatement evaluates the classes directly:
// (LS|LS) -> LS block, (LS|SL) -> LL block, (SL|LS) -> SS block, and fills
// the SL block by the final conjugation of BRTFAST (:17643-17654):
// BXCH(J,I) = conj(BXCH(I,J)), I large, J small.
void breit_full(const Basis &b, const Opts &o, bool gaunt, const Mat &D, Mat &BX) {
  for (int j = 0; j < b.ndim; ++j)
    for (int i = 0; i < b.ndim; ++i) BX(i, j) = 0.0;
  std::deque<EBlockQ> ecache;
  std::vector<int> ekey;
  auto eblock = [&](int c1, int l1, int c2, int l2, int sm) -> const EBlockQ & {
    int key = (((c1 * 16 + l1) * 1024 + c2) * 16 + l2) * 2 + sm;
    for (size_t i = 0; i < ekey.size(); ++i)
      if (ekey[i] == key) return ecache[i];
    ekey.push_back(key);
    ecache.push_back(make_eblock_q(b, c1, l1, c2, l2, sm != 0));
    return ecache.back();
  };
  const int classes[3][2] = {{0, 0}, {0, 1}, {1, 0}};  // 0 = LS, 1 = SL
  for (int ca = 0; ca < b.ncnt; ++ca)
  for (int cb = 0; cb < b.ncnt; ++cb)
  for (int cc = 0; cc < b.ncnt; ++cc)
  for (int cd = 0; cd < b.ncnt; ++cd) {
    int mcnt = ncntrs(ca, cb, cc, cd);
    if (mcnt == 1 && o.racah1) continue;
    if (mcnt != 1 && o.ilev < 3) continue;
    for (int lA = 0; lA <= b.lmax[ca]; ++lA)
    for (int lB = 0; lB <= b.lmax[cb]; ++lB)
    for (int lC = 0; lC <= b.lmax[cc]; ++lC)
    for (int lD = 0; lD <= b.lmax[cd]; ++lD) {
      if (mcnt == 1 && ((lA + lB) % 2) != ((lC + lD) % 2)) continue;
      int lq[4] = {lA, lB, lC, lD};
      for (const auto &cl : classes) {
        int t1 = cl[0], t2 = cl[1];
        const EBlockQ &Eab = eblock(ca, lA, cb, lB, t1);
        const EBlockQ &Ecd = eblock(cc, lC, cd, lD, t2);
        int degab = lA + lB + 1, degcd = lC + lD + 1, ncd = Ecd.nt;
        const double *A = &b.xyz[3 * ca], *B = &b.xyz[3 * cb];
        const double *Cc = &b.xyz[3 * cc], *Dd = &b.xyz[3 * cd];
        // Fock offsets: LS puts a in the large and b in the small block
        int oa = t1 ? b.nskp : 0, ob = t1 ? 0 : b.nskp;
        int oc = t2 ? b.nskp : 0, od = t2 ? 0 : b.nskp;
        std::vector<double> Wt;
        std::vector<cplx> g11(3 * ncd), g21(3 * ncd);
        for (int i = 0; i < Eab.na; ++i)
        for (int j = 0; j < Eab.nb; ++j) {
          double ei = b.ex[ca][lA][i], ej = b.ex[cb][lB][j], eij = ei + ej;
          double P[3];
          for (int x = 0; x < 3; ++x) P[x] = (A[x] * ei + B[x] * ej) / eij;
          int ij = i * Eab.nb + j;
          for (int k = 0; k < Ecd.na; ++k)
          for (int l = 0; l < Ecd.nb; ++l) {
            double ek = b.ex[cc][lC][k], el = b.ex[cd][lD][l], ekl = ek + el;
            double Q[3];
            for (int x = 0; x < 3; ++x) Q[x] = (Cc[x] * ek + Dd[x] * el) / ekl;
            bii_table(P, eij, Q, ekl, degab, degcd, gaunt, Wt);
            int kl = k * Ecd.nb + l;
            for (int ia = 0; ia < Eab.nlab_a; ++ia)
            for (int ib = 0; ib < Eab.nlab_b; ++ib) {
              const Label &LA = Eab.la[ia], &LB = Eab.lb[ib];
              bii_first(Eab, ia, ib, ij, Wt, ncd, g11.data(), g21.data());
              int na[2] = {b.lrge[ca][LA.ka][2 * LA.ma - 2] + oa + i,
                           b.lrge[ca][LA.ka][2 * LA.ma - 1] + oa + i};
              int nb[2] = {b.lrge[cb][LB.ka][2 * LB.ma - 2] + ob + j,
                           b.lrge[cb][LB.ka][2 * LB.ma - 1] + ob + j};
              for (int ic = 0; ic < Ecd.nlab_a; ++ic)
              for (int id = 0; id < Ecd.nlab_b; ++id) {
                const Label &LC = Ecd.la[ic], &LD = Ecd.lb[id];
                Label quad[4] = {LA, LB, LC, LD};
                if (!label_rules(o, mcnt, quad, lq, true)) continue;
                double pab = phase_breit(LA.kq, LA.ma, LB.kq, LB.ma);
                double pcd = phase_breit(LC.kq, LC.ma, LD.kq, LD.ma);
                Eri16 rr;
                bii_second(g11.data(), g21.data(), Ecd, ic, id, kl, ncd, pab, pcd, rr);
                int nc[2] = {b.lrge[cc][LC.ka][2 * LC.ma - 2] + oc + k,
                             b.lrge[cc][LC.ka][2 * LC.ma - 1] + oc + k};
                int nd[2] = {b.lrge[cd][LD.ka][2 * LD.ma - 2] + od + l,
                             b.lrge[cd][LD.ka][2 * LD.ma - 1] + od + l};
                digest_x(rr, na, nb, nc, nd, D, BX, o.isym);
              }
            }
          }
        }
      }
    }
  }
  for (int i = 0; i < b.nskp; ++i)
    for (int j = b.nskp; j < b.ndim; ++j) BX(j, i) = std::conj(BX(i, j));
}

// ---------------------------------------------------------------------------
// One-electron matrices (ONEEL bertha-scf.f:6996-7990, OVRLP :6683)
// ---------------------------------------------------------------------------
const double CLIGHT = 137.035999084;  // speed of light (bertha-scf.f:974)

// The four m-sign combinations of a one-electron element from sets
// (-|ma|,-|mb|) and (+|ma|,-|mb|): (-,+) = -PHS conj(+,-), (+,+) = PHS conj(-,-)
// (ONEEL :7106-7109, PHS as the Coulomb pair phase).
void put4(Mat &M, const int ra[2], const int cb[2], cplx x11, cplx x21, double phs) {
  M(ra[0], cb[0]) = x11;
  M(ra[1], cb[0]) = x21;
  M(ra[0], cb[1]) = -phs * std::conj(x21);
  M(ra[1], cb[1]) = phs * std::conj(x11);
}

// Nuclear attraction of one primitive pair density with E-coefficients e
// (degree deg) to every nucleus: point (xi = 0; APH = p, PNC = 2 pi Z/p) or
// Gaussian (APH = p xi/(p+xi), PNC = 2 pi Z sqrt(xi/(p+xi))/p), ONEEL
// :7250-7330.  Returns -sum_C PNC sum_tuv E_tuv R_tuv(APH, C - P).
cplx nuc_attr(const cplx *e, int deg, double p, const double *P, const Basis &b,
              const double *znuc, const double *xi) {
  cplx v(0.0);
  std::vector<double> R(ntuv(deg));
  for (int c = 0; c < b.ncnt; ++c) {
    double cp[3];
    for (int x = 0; x < 3; ++x) cp[x] = b.xyz[3 * c + x] - P[x];
    double aph, pnc;
    if (xi[c] > 0.0) {
      aph = p * xi[c] / (p + xi[c]);
      pnc = 2.0 * PI * znuc[c] * std::sqrt(xi[c] / (p + xi[c])) / p;
    } else {
      aph = p;
      pnc = 2.0 * PI * znuc[c] / p;
    }
    rints(cp, aph, deg, R.data());
    cplx acc(0.0);
    for (int k = 0; k < ntuv(deg); ++k) acc += e[k] * R[k];
    v -= pnc * acc;
  }
  return v;
}

// OVLP, HNUC = V (LL), V - 2c^2 S (SS), HKIN = c sqrt((2l+3) alpha) S_SS
// couplings (ONEEL parts 1-4) or, for NORL, the non-relativistic kinetic
// matrix (:7420-7470).  Every ordered shell pair is computed directly.
void oneel_full(const Basis &b, int hmlt, const double *znuc, const double *xi, Mat &S, Mat &V,
                Mat &T) {
  for (int j = 0; j < b.ndim; ++j)
    for (int i = 0; i < b.ndim; ++i) S(i, j) = V(i, j) = T(i, j) = 0.0;
  const Cart &C = cart();
  bool norl = hmlt == 0;
  for (int ca = 0; ca < b.ncnt; ++ca)
  for (int cb = 0; cb < b.ncnt; ++cb)
  for (int lA = 0; lA <= b.lmax[ca]; ++lA)
  for (int lB = 0; lB <= b.lmax[cb]; ++lB) {
    std::vector<Label> la = labels_for(lA), lb = labels_for(lB);
    const double *A = &b.xyz[3 * ca], *B = &b.xyz[3 * cb];
    for (size_t ia = 0; ia < la.size(); ++ia)
    for (size_t ib = 0; ib < lb.size(); ++ib) {
      double phs = phase_pair(la[ia].kq, la[ia].ma, lb[ib].kq, lb[ib].ma);
      int mqa = 2 * la[ia].ma - 1, mqb = 2 * lb[ib].ma - 1;
      for (size_t i = 0; i < b.ex[ca][lA].size(); ++i)
      for (size_t j = 0; j < b.ex[cb][lB].size(); ++j) {
        double ea = b.ex[ca][lA][i], eb = b.ex[cb][lB][j], p = ea + eb;
        double P[3];
        for (int x = 0; x < 3; ++x) P[x] = (A[x] * ea + B[x] * eb) / p;
        double eroot = std::pow(PI / p, 1.5);
        int ra[2] = {b.lrge[ca][la[ia].ka][2 * la[ia].ma - 2] + (int)i,
                     b.lrge[ca][la[ia].ka][2 * la[ia].ma - 1] + (int)i};
        int cl[2] = {b.lrge[cb][lb[ib].ka][2 * lb[ib].ma - 2] + (int)j,
                     b.lrge[cb][lb[ib].ka][2 * lb[ib].ma - 1] + (int)j};
        HVec l11 = eq_pair(la[ia].kq, -mqa, ea, A, lb[ib].kq, -mqb, eb, B, false);
        HVec l21 = eq_pair(la[ia].kq, mqa, ea, A, lb[ib].kq, -mqb, eb, B, false);
        put4(S, ra, cl, eroot * l11[0], eroot * l21[0], phs);
        put4(V, ra, cl, nuc_attr(l11.data(), lA + lB, p, P, b, znuc, xi),
             nuc_attr(l21.data(), lA + lB, p, P, b, znuc, xi), phs);
        if (norl) {
          double PB[3] = {P[0] - B[0], P[1] - B[1], P[2] - B[2]};
          double pb2 = PB[0] * PB[0] + PB[1] * PB[1] + PB[2] * PB[2];
          double e0 = eb * (2 * lB + 3) - 2.0 * eb * eb * pb2 - 3.0 * eb * eb / p;
          double e1 = 4.0 * eb * eb;
          cplx t[2];
          const HVec *ee[2] = {&l11, &l21};
          for (int s2 = 0; s2 < 2; ++s2) {
            const HVec &e = *ee[s2];
            cplx tr = e0 * e[0];
            if (lA + lB >= 1)
              tr -= e1 * (PB[0] * e[C.idx[1][0][0]] + PB[1] * e[C.idx[0][1][0]] +
                          PB[2] * e[C.idx[0][0][1]]);
            if (lA + lB >= 2)
              tr -= e1 * (e[C.idx[2][0][0]] + e[C.idx[0][2][0]] + e[C.idx[0][0][2]]);
            t[s2] = eroot * tr;
          }
          put4(T, ra, cl, t[0], t[1], phs);
          continue;
        }
        HVec s11 = eq_pair(la[ia].kq, -mqa, ea, A, lb[ib].kq, -mqb, eb, B, true);
        HVec s21 = eq_pair(la[ia].kq, mqa, ea, A, lb[ib].kq, -mqb, eb, B, true);
        int rs[2] = {ra[0] + b.nskp, ra[1] + b.nskp}, cs[2] = {cl[0] + b.nskp, cl[1] + b.nskp};
        cplx ss11 = eroot * s11[0], ss21 = eroot * s21[0];
        put4(S, rs, cs, ss11, ss21, phs);
        double cv2 = 2.0 * CLIGHT * CLIGHT;
        put4(V, rs, cs, nuc_attr(s11.data(), lA + lB + 2, p, P, b, znuc, xi) - cv2 * ss11,
             nuc_attr(s21.data(), lA + lB + 2, p, P, b, znuc, xi) - cv2 * ss21, phs);
        double fsl = CLIGHT * std::sqrt((2 * lB + 3) * eb);  // T(a_S, b_L)
        double fls = CLIGHT * std::sqrt((2 * lA + 3) * ea);  // T(a_L, b_S)
        put4(T, rs, cl, fsl * ss11, fsl * ss21, phs);
        put4(T, ra, cs, fls * ss11, fls * ss21, phs);
      }
    }
  }
}

Basis make_basis(int ncnt, const double *xyz, const int *lmax, const int *nfn,
                 const double *ex, int maxl1, int maxbs, bool norl) {
  Basis b;
  b.ncnt = ncnt;
  b.xyz.assign(xyz, xyz + 3 * ncnt);
  b.lmax.assign(lmax, lmax + ncnt);
  b.ex.resize(ncnt);
  for (int c = 0; c < ncnt; ++c) {
    b.ex[c].resize(lmax[c] + 1);
    for (int l = 0; l <= lmax[c]; ++l) {
      int n = nfn[c * maxl1 + l];
      for (int i = 0; i < n; ++i)
        b.ex[c][l].push_back(ex[((size_t)c * maxl1 + l) * maxbs + i]);
    }
  }
  fock_layout(b, norl);
  return b;
}

}  // namespace

// ---------------------------------------------------------------------------
// C interface used by the tests (ctypes).  Complex matrices are interleaved
// (re, im) doubles, column-major with leading dimension ld.
// ---------------------------------------------------------------------------
extern "C" {

int orc_boys(double T, int lam, double *F) {
  if (lam < 0 || lam > MAXL) return 1;
  boys(T, lam, F);
  return 0;
}

int orc_rints(const double *qp, double alpha, int lam, double *R) {
  if (lam < 0 || lam > MAXL) return 1;
  rints(qp, alpha, lam, R);
  return 0;
}

// Hermite index of (t,u,v) in CARTIND order
int orc_cart_index(int t, int u, int v) { return cart().idx[t][u][v]; }

// E-coefficients for one primitive pair; out receives ntuv(degree) complex.
int orc_eq_pair(int ka, int mqa, double ea, const double *A, int kb, int mqb,
                double eb, const double *B, int small, double *out) {
  HVec h = eq_pair(ka, mqa, ea, A, kb, mqb, eb, B, small != 0);
  for (size_t k = 0; k < h.size(); ++k) {
    out[2 * k] = h[k].real();
    out[2 * k + 1] = h[k].imag();
  }
  return int(h.size());
}

// Fock layout: writes LRGE offsets lrge[(cnt*(2*maxl+2) + ka)*28 + mqn-1]
// (ka 1-based, mqn-1 = 2|m|-1 + sign) and returns NDIM.
int orc_fock_layout(int ncnt, const double *xyz, const int *lmax,
                    const int *nfn, const double *ex, int maxl1, int maxbs,
                    int norl, int *lrge_out, int *nskp_out) {
  Basis b = make_basis(ncnt, xyz, lmax, nfn, ex, maxl1, maxbs, norl != 0);
  int nk = 2 * (maxl1 - 1) + 2;
  for (int c = 0; c < ncnt; ++c)
    for (int ka = 0; ka < (int)b.lrge[c].size(); ++ka)
      for (int m = 0; m < 28; ++m)
        lrge_out[((size_t)c * nk + ka) * 28 + m] =
            m < (int)b.lrge[c][ka].size() ? b.lrge[c][ka][m] : -1;
  *nskp_out = b.nskp;
  return b.ndim;
}

// Oracle context for explicit shell-quartet lists (the ERI microbenchmark):
// shells in the order centre, l, exponent; E-coefficients prepared once.
struct OrcCtx {
  Basis b;
  struct Sh { int c, l, i; };
  std::vector<Sh> sh;
  std::vector<std::vector<HVec>> eq;  // [pair*2+comp][lab_a][lab_b][set] flattened
  std::vector<char> have;
};

// One shell quartet: all label pairs, 16 m-signs, batch types 1 and 5.
void orc_one_quartet(const OrcCtx &o, const int *q, int t1, int t2, const Mat &D,
                     Mat &GD, Mat &GX, bool atomic) {
  const Cart &C = cart();
  const OrcCtx::Sh &A = o.sh[q[0]], &B = o.sh[q[1]], &Cc = o.sh[q[2]], &Dd = o.sh[q[3]];
  const Basis &b = o.b;
  size_t ns = o.sh.size();
  const std::vector<HVec> &Eab = o.eq[((size_t)q[0] * ns + q[1]) * 2 + t1];
  const std::vector<HVec> &Ecd = o.eq[((size_t)q[2] * ns + q[3]) * 2 + t2];
  std::vector<Label> la = labels_for(A.l), lb = labels_for(B.l);
  std::vector<Label> lc = labels_for(Cc.l), ld = labels_for(Dd.l);
  int degab = A.l + B.l + 2 * t1, degcd = Cc.l + Dd.l + 2 * t2, lam = degab + degcd;
  int nab = ntuv(degab), ncd = ntuv(degcd);
  double ei = b.ex[A.c][A.l][A.i], ej = b.ex[B.c][B.l][B.i];
  double ek = b.ex[Cc.c][Cc.l][Cc.i], el = b.ex[Dd.c][Dd.l][Dd.i];
  double eij = ei + ej, ekl = ek + el, qp[3];
  for (int x = 0; x < 3; ++x)
    qp[x] = (b.xyz[3 * Cc.c + x] * ek + b.xyz[3 * Dd.c + x] * el) / ekl -
            (b.xyz[3 * A.c + x] * ei + b.xyz[3 * B.c + x] * ej) / eij;
  std::vector<double> R(ntuv(lam));
  rints(qp, eij * ekl / (eij + ekl), lam, R.data());
  double pre = 2.0 * PI52 / (std::sqrt(eij + ekl) * eij * ekl);
  for (double &r : R) r *= pre;
  int oab = t1 ? b.nskp : 0, ocd = t2 ? b.nskp : 0;
  std::vector<cplx> g11(ncd), g21(ncd);
  for (size_t ia = 0; ia < la.size(); ++ia)
  for (size_t ib = 0; ib < lb.size(); ++ib) {
    const HVec &e11 = Eab[(ia * lb.size() + ib) * 2], &e21 = Eab[(ia * lb.size() + ib) * 2 + 1];
    for (int qq = 0; qq < ncd; ++qq) {
      cplx x(0), y(0);
      for (int s = 0; s < nab; ++s) {
        double rv = R[C.idx[C.t[s] + C.t[qq]][C.u[s] + C.u[qq]][C.v[s] + C.v[qq]]];
        x += e11[s] * rv;
        y += e21[s] * rv;
      }
      g11[qq] = x;
      g21[qq] = y;
    }
    int na[2] = {b.lrge[A.c][la[ia].ka][2 * la[ia].ma - 2] + oab + A.i,
                 b.lrge[A.c][la[ia].ka][2 * la[ia].ma - 1] + oab + A.i};
    int nb[2] = {b.lrge[B.c][lb[ib].ka][2 * lb[ib].ma - 2] + oab + B.i,
                 b.lrge[B.c][lb[ib].ka][2 * lb[ib].ma - 1] + oab + B.i};
    for (size_t ic = 0; ic < lc.size(); ++ic)
    for (size_t id = 0; id < ld.size(); ++id) {
      Eri16 rr;
      double pab = phase_pair(la[ia].kq, la[ia].ma, lb[ib].kq, lb[ib].ma);
      double pcd = phase_pair(lc[ic].kq, lc[ic].ma, ld[id].kq, ld[id].ma);
      const HVec &f11 = Ecd[(ic * ld.size() + id) * 2], &f21 = Ecd[(ic * ld.size() + id) * 2 + 1];
      second_contraction(g11.data(), g21.data(), f11.data(), f21.data(), ncd, pab, pcd, rr);
      int nc[2] = {b.lrge[Cc.c][lc[ic].ka][2 * lc[ic].ma - 2] + ocd + Cc.i,
                   b.lrge[Cc.c][lc[ic].ka][2 * lc[ic].ma - 1] + ocd + Cc.i};
      int nd[2] = {b.lrge[Dd.c][ld[id].ka][2 * ld[id].ma - 2] + ocd + Dd.i,
                   b.lrge[Dd.c][ld[id].ka][2 * ld[id].ma - 1] + ocd + Dd.i};
      if (!atomic) {
        digest(rr, na, nb, nc, nd, D, GD, GX, 0);
      } else {
        for (int sa = 0; sa < 2; ++sa)
        for (int sb = 0; sb < 2; ++sb)
        for (int sc = 0; sc < 2; ++sc)
        for (int sd = 0; sd < 2; ++sd) {
          cplx v = rr.v[8 * sa + 4 * sb + 2 * sc + sd];
          cplx j = v * D(nc[sc], nd[sd]), k = v * D(nc[sc], nb[sb]);
          double *pj = reinterpret_cast<double *>(&GD(na[sa], nb[sb]));
          double *pk = reinterpret_cast<double *>(&GX(na[sa], nd[sd]));
#ifdef _OPENMP
#pragma omp atomic
#endif
          pj[0] += j.real();
#ifdef _OPENMP
#pragma omp atomic
#endif
          pj[1] += j.imag();
#ifdef _OPENMP
#pragma omp atomic
#endif
          pk[0] += k.real();
#ifdef _OPENMP
#pragma omp atomic
#endif
          pk[1] += k.imag();
        }
      }
    }
  }
}

// All spinor integrals of one primitive quartet: shells given by centre,
// l and exponent; t1/t2 select LL (0) or SS (1) for the ab and cd pairs.
// out: [lab_a][lab_b][lab_c][lab_d][16] complex with labels ordered as
// labels_for(l) (kappa=l then kappa=-l-1, |m| ascending); returns the count.
int orc_eri_quartet(const double *xyz4, const int *l4, const double *ex4,
                    int t1, int t2, double *out) {
  Basis b;
  b.ncnt = 4;
  b.xyz.assign(xyz4, xyz4 + 12);
  b.lmax.assign(4, 0);
  b.ex.assign(4, {});
  for (int c = 0; c < 4; ++c) {
    b.lmax[c] = l4[c];
    b.ex[c].assign(l4[c] + 1, {});
    b.ex[c][l4[c]].push_back(ex4[c]);
  }
  EBlock Eab = make_eblock(b, 0, l4[0], 1, l4[1], t1 != 0);
  EBlock Ecd = make_eblock(b, 2, l4[2], 3, l4[3], t2 != 0);
  const Cart &C = cart();
  int lam = (l4[0] + l4[1] + 2 * t1) + (l4[2] + l4[3] + 2 * t2);
  double eij = ex4[0] + ex4[1], ekl = ex4[2] + ex4[3], qp[3];
  for (int x = 0; x < 3; ++x)
    qp[x] = (xyz4[6 + x] * ex4[2] + xyz4[9 + x] * ex4[3]) / ekl -
            (xyz4[x] * ex4[0] + xyz4[3 + x] * ex4[1]) / eij;
  std::vector<double> R(ntuv(lam));
  rints(qp, eij * ekl / (eij + ekl), lam, R.data());
  double pre = 2.0 * PI52 / (std::sqrt(eij + ekl) * eij * ekl);
  for (double &r : R) r *= pre;
  int n = 0;
  std::vector<cplx> g11(Ecd.nt), g21(Ecd.nt);
  for (int ia = 0; ia < Eab.nlab_a; ++ia)
  for (int ib = 0; ib < Eab.nlab_b; ++ib) {
    const cplx *e11 = Eab.at(ia, ib, 0, 0), *e21 = Eab.at(ia, ib, 1, 0);
    for (int q = 0; q < Ecd.nt; ++q) {
      cplx a(0), bq(0);
      for (int s = 0; s < Eab.nt; ++s) {
        double rv = R[C.idx[C.t[s] + C.t[q]][C.u[s] + C.u[q]][C.v[s] + C.v[q]]];
        a += e11[s] * rv;
        bq += e21[s] * rv;
      }
      g11[q] = a;
      g21[q] = bq;
    }
    for (int ic = 0; ic < Ecd.nlab_a; ++ic)
    for (int id = 0; id < Ecd.nlab_b; ++id) {
      Eri16 rr;
      double pab = phase_pair(Eab.la[ia].kq, Eab.la[ia].ma, Eab.lb[ib].kq,
                              Eab.lb[ib].ma);
      double pcd = phase_pair(Ecd.la[ic].kq, Ecd.la[ic].ma, Ecd.lb[id].kq,
                              Ecd.lb[id].ma);
      second_contraction(g11.data(), g21.data(), Ecd.at(ic, id, 0, 0),
                         Ecd.at(ic, id, 1, 0), Ecd.nt, pab, pcd, rr);
      for (int s = 0; s < 16; ++s) {
        out[2 * n] = rr.v[s].real();
        out[2 * n + 1] = rr.v[s].imag();
        ++n;
      }
    }
  }
  return n;
}

void *orc_ctx_new(int ncnt, const double *xyz, const int *lmax, const int *nfn,
                  const double *ex, int maxl1, int maxbs, int hmlt) {
  OrcCtx *o = new OrcCtx();
  o->b = make_basis(ncnt, xyz, lmax, nfn, ex, maxl1, maxbs, hmlt == 0);
  for (int c = 0; c < ncnt; ++c)
    for (int l = 0; l <= o->b.lmax[c]; ++l)
      for (int i = 0; i < (int)o->b.ex[c][l].size(); ++i) o->sh.push_back({c, l, i});
  size_t ns = o->sh.size();
  o->eq.assign(ns * ns * 2, {});
  o->have.assign(ns * ns * 2, 0);
  return o;
}

void orc_ctx_free(void *h) { delete (OrcCtx *)h; }

// Prepare E-coefficients of every shell pair used by the quartet list.
int orc_ctx_prepare(void *h, const int *quart, long long n, int t1, int t2) {
  OrcCtx &o = *(OrcCtx *)h;
  std::vector<std::pair<int, int>> need;
  size_t ns = o.sh.size();
  std::vector<char> mark(ns * ns * 2, 0);
  for (long long i = 0; i < n; ++i) {
    size_t k1 = ((size_t)quart[4 * i] * ns + quart[4 * i + 1]) * 2 + t1;
    size_t k2 = ((size_t)quart[4 * i + 2] * ns + quart[4 * i + 3]) * 2 + t2;
    if (!mark[k1] && !o.have[k1]) { mark[k1] = 1; need.push_back({(int)(k1 / 2), t1}); }
    if (!mark[k2] && !o.have[k2]) { mark[k2] = 1; need.push_back({(int)(k2 / 2), t2}); }
  }
  std::vector<std::vector<HVec>> tmp(need.size());
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic)
#endif
  for (long long i = 0; i < (long long)need.size(); ++i) {
    int pr = need[i].first;
    const OrcCtx::Sh &A = o.sh[pr / ns], &B = o.sh[pr % ns];
    std::vector<Label> la = labels_for(A.l), lb = labels_for(B.l);
    for (size_t ia = 0; ia < la.size(); ++ia)
      for (size_t ib = 0; ib < lb.size(); ++ib)
        for (int set = 0; set < 2; ++set) {
          int mqa = (set == 0 ? -1 : 1) * (2 * la[ia].ma - 1);
          int mqb = -(2 * lb[ib].ma - 1);
          tmp[i].push_back(eq_pair(la[ia].kq, mqa, o.b.ex[A.c][A.l][A.i], &o.b.xyz[3 * A.c],
                                   lb[ib].kq, mqb, o.b.ex[B.c][B.l][B.i],
                                   &o.b.xyz[3 * B.c], need[i].second != 0));
        }
  }
  for (size_t i = 0; i < need.size(); ++i) {
    size_t key = (size_t)need[i].first * 2 + need[i].second;
    o.eq[key] = std::move(tmp[i]);
    o.have[key] = 1;
  }
  return (int)need.size();
}

// Digest an explicit quartet list (adds into gd/gx, batch types 1 and 5),
// with nthreads OpenMP threads (atomic accumulation when > 1).
int orc_ctx_quartets(void *h, const int *quart, long long n, int t1, int t2,
                     const double *dent, int ldd, double *gd, double *gx, int ldf,
                     int nthreads) {
  OrcCtx &o = *(OrcCtx *)h;
  orc_ctx_prepare(h, quart, n, t1, t2);
  Mat D{(cplx *)dent, ldd}, GD{(cplx *)gd, ldf}, GX{(cplx *)gx, ldf};
  bool atomic = nthreads > 1;
#ifdef _OPENMP
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
#endif
  for (long long i = 0; i < n; ++i) {
    Mat gdl = GD, gxl = GX;
    orc_one_quartet(o, &quart[4 * i], t1, t2, D, gdl, gxl, atomic);
  }
  return 0;
}

// Spinor overlap E-coefficients psi_a^+ sigma_q psi_b for any component
// pair (sa, sb: 0 large, 1 small) and q = 0 (unit), 1..3 (x, y, z).
int orc_eq_pair_q(int ka, int mqa, double ea, const double *A, int kb, int mqb,
                  double eb, const double *B, int sa, int sb, int iq, double *out) {
  HVec h = eq_pair_q(ka, mqa, ea, A, kb, mqb, eb, B, sa != 0, sb != 0, iq);
  for (size_t k = 0; k < h.size(); ++k) {
    out[2 * k] = h[k].real();
    out[2 * k + 1] = h[k].imag();
  }
  return int(h.size());
}

// Breit kernel W_ij at Hermite index (t,u,v) for PQ = qp and exponent alpha
// with PRE = 1 (R-integrals only); out: 3x3 row-major.
int orc_breit_kernel(const double *qp, double alpha, int t, int u, int v, int gaunt,
                     double *out) {
  int lam = t + u + v + 2;
  std::vector<double> R(ntuv(lam));
  rints(qp, alpha, lam, R.data());
  double W[3][3];
  breit_kernel(R.data(), qp, alpha, t, u, v, gaunt != 0, W);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) out[3 * i + j] = W[i][j];
  return 0;
}

// All Breit (or Gaunt) integrals of one primitive quartet; t1/t2 select LS
// (0) or SL (1) for the ab and cd pairs.  out as orc_eri_quartet.
int orc_bii_quartet(const double *xyz4, const int *l4, const double *ex4, int t1, int t2,
                    int gaunt, double *out) {
  Basis b;
  b.ncnt = 4;
  b.xyz.assign(xyz4, xyz4 + 12);
  b.lmax.assign(4, 0);
  b.ex.assign(4, {});
  for (int c = 0; c < 4; ++c) {
    b.lmax[c] = l4[c];
    b.ex[c].assign(l4[c] + 1, {});
    b.ex[c][l4[c]].push_back(ex4[c]);
  }
  EBlockQ Eab = make_eblock_q(b, 0, l4[0], 1, l4[1], t1 != 0);
  EBlockQ Ecd = make_eblock_q(b, 2, l4[2], 3, l4[3], t2 != 0);
  double P[3], Q[3];
  for (int x = 0; x < 3; ++x) {
    P[x] = (xyz4[x] * ex4[0] + xyz4[3 + x] * ex4[1]) / (ex4[0] + ex4[1]);
    Q[x] = (xyz4[6 + x] * ex4[2] + xyz4[9 + x] * ex4[3]) / (ex4[2] + ex4[3]);
  }
  std::vector<double> Wt;
  bii_table(P, ex4[0] + ex4[1], Q, ex4[2] + ex4[3], l4[0] + l4[1] + 1, l4[2] + l4[3] + 1,
            gaunt != 0, Wt);
  int ncd = Ecd.nt, n = 0;
  std::vector<cplx> g11(3 * ncd), g21(3 * ncd);
  for (int ia = 0; ia < Eab.nlab_a; ++ia)
  for (int ib = 0; ib < Eab.nlab_b; ++ib) {
    bii_first(Eab, ia, ib, 0, Wt, ncd, g11.data(), g21.data());
    for (int ic = 0; ic < Ecd.nlab_a; ++ic)
    for (int id = 0; id < Ecd.nlab_b; ++id) {
      double pab = phase_breit(Eab.la[ia].kq, Eab.la[ia].ma, Eab.lb[ib].kq, Eab.lb[ib].ma);
      double pcd = phase_breit(Ecd.la[ic].kq, Ecd.la[ic].ma, Ecd.lb[id].kq, Ecd.lb[id].ma);
      Eri16 rr;
      bii_second(g11.data(), g21.data(), Ecd, ic, id, 0, ncd, pab, pcd, rr);
      for (int s = 0; s < 16; ++s) {
        out[2 * n] = rr.v[s].real();
        out[2 * n + 1] = rr.v[s].imag();
        ++n;
      }
    }
  }
  return n;
}

// Closed-shell multi-centre Breit exchange matrix (BRTFAST, NOPN = 0).
int orc_brtfast(int ncnt, const double *xyz, const int *lmax, const int *nfn,
                const double *ex, int maxl1, int maxbs, int isym, int ilev, int racah1,
                int gaunt, const double *dent, int ldd, double *bxch, int ldf) {
  Basis b = make_basis(ncnt, xyz, lmax, nfn, ex, maxl1, maxbs, false);
  Opts o{ilev, isym, 2, racah1, 0, 0};
  Mat D{(cplx *)dent, ldd}, BX{(cplx *)bxch, ldf};
  breit_full(b, o, gaunt != 0, D, BX);
  return b.ndim;
}

// One-electron matrices OVLP, HNUC, HKIN of ONEEL (xi = 0: point nucleus).
int orc_oneel(int ncnt, const double *xyz, const int *lmax, const int *nfn, const double *ex,
              int maxl1, int maxbs, int hmlt, const double *znuc, const double *xi,
              double *ovlp, double *hnuc, double *hkin, int ldf) {
  Basis b = make_basis(ncnt, xyz, lmax, nfn, ex, maxl1, maxbs, hmlt == 0);
  Mat S{(cplx *)ovlp, ldf}, V{(cplx *)hnuc, ldf}, T{(cplx *)hkin, ldf};
  oneel_full(b, hmlt, znuc, xi, S, V, T);
  return b.ndim;
}

int orc_ndim(void *h, int *nskp) {
  OrcCtx &o = *(OrcCtx *)h;
  *nskp = o.b.nskp;
  return o.b.ndim;
}

// Full-mode multi-centre Coulomb Fock build (CLMFAST with INTSYM=.FALSE.).
int orc_clmfast(int ncnt, const double *xyz, const int *lmax, const int *nfn,
                const double *ex, int maxl1, int maxbs, int hmlt, int isym,
                int ilev, int racah1, const double *dent, int ldd,
                double *gdir, double *gxch, int ldf) {
  Basis b = make_basis(ncnt, xyz, lmax, nfn, ex, maxl1, maxbs, hmlt == 0);
  Opts o{ilev, isym, hmlt, racah1, 0, 0};
  Mat D{(cplx *)dent, ldd}, GD{(cplx *)gdir, ldf}, GX{(cplx *)gxch, ldf};
  fock_full(b, o, D, GD, GX);
  return b.ndim;
}

}  // extern "C"

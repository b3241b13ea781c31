// GB300 (sm_103a) multi-centre Dirac-Coulomb Fock build behind the C ABI of
// include/bertha_gpu.h.  FP64 throughout (the drop-in precision of the
// reference, bertha-scf.f CLMFAST/ERIFAST/CLMMTG/CLMMTZ).
//
// Device work:
//   k_eqgen     spinor E-coefficients of every shell pair, LL and SS
//               (EQSAVE/EQLL/EQSS, bertha-scf.f:32984-36900)
//   k_quartet   one CTA per ordered shell quartet: Boys function in the
//               reference's four regimes (FUNFM :32465), Hermite R-integrals
//               (RMAKE :31900) in shared memory, first and second contraction
//               of ERIFAST (:12676-13126) over ab-label chunks, and the J/K
//               digestion of CLMMTG/CLMMTZ batch types 1 and 5 into shared
//               accumulators flushed with one atomic per element.
//   k_zero      clears the outputs (CLMFAST zeroes GDIR/GXCH, :11592).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "bertha_gpu.h"

// Scratch of bertha_gpu_quartets_noalloc: the double-float copy of the
// density, BG_NOALLOC_MAX_NDIM^2 float4 (16 MiB), resident on every GPU that
// loads the library until the process exits.  Host code must not pass this
// name to a kernel: it only names a host-side stand-in; the device address
// comes from cudaGetSymbolAddress (noalloc_scratch below).
static __device__ __align__(256) float4
    g_noalloc_density[(size_t)BG_NOALLOC_MAX_NDIM * BG_NOALLOC_MAX_NDIM];

namespace {

__host__ __device__ constexpr int ntuv(int L) { return L < 0 ? 0 : (L + 1) * (L + 2) * (L + 3) / 6; }

constexpr int MAXLB = BG_MAX_L;           // basis l
constexpr int MAXLAB = 2 * MAXLB + 1;     // spinor labels (kappa,|m|) per shell
constexpr int MAXSP = 2 * MAXLAB;         // spinors per shell and component
constexpr int MAXDEGE = 2 * MAXLB + 2;    // E degree (SS)
constexpr int MAXLAM = 2 * MAXDEGE;       // R order (SS|SS)
constexpr int NTE = ntuv(MAXDEGE);        // 165
constexpr int NTR = ntuv(MAXLAM);         // 969
constexpr int CHUNK = 5;                  // ab labels per first-contraction pass (at N = 165)
constexpr int QT64 = 128;                 // k_quartet, k_breit: four 128-thread CTAs per SM

__constant__ signed char c_t[NTR], c_u[NTR], c_v[NTR];

// Hermite index in CARTIND order (bertha-scf.f:2651): lambda, then t, then u.
__host__ __device__ inline int hidx(int t, int u, int v) {
  int L = t + u + v;
  return ntuv(L - 1) + t * (L + 1) - (t * (t - 1)) / 2 + u;
}

struct Shell {
  double x, y, z, alpha;
  int l, cnt, ibas;
  int inst;             // instance of a batched build (0 for a single context)
  int prow;             // pair-table row: pair (this, b) is pe[prow + b]
  int pad;
  int fock[MAXLAB][2];  // large-component Fock index of m<0 / m>0
};

// Placement of one instance's matrices in a batched build: element (i, j)
// of its D, J and K sits at off + i + ld*j (complex units).
struct Inst {
  long long off;
  int ld, nskp;
};

struct PairE {
  long long off[2];  // E offset (complex units) for LL and SS, -1 if absent
  int kexp;          // power-of-two scale of the double-float copy (see k_econv)
  int pad;
};

// complex helpers
__host__ __device__ inline double2 cadd(double2 a, double2 b) {
  return make_double2(a.x + b.x, a.y + b.y);
}
__host__ __device__ inline double2 cscale(double2 a, double s) {
  return make_double2(a.x * s, a.y * s);
}

// ---------------------------------------------------------------------------
// E-coefficient generation (Saunders recursion of EVRS/ESTEPLM/ESTEPL/ESTEPN)
// ---------------------------------------------------------------------------
struct Geo {
  double p, PA[3], PB[3], PA2, PB2, rkab;
};

// out += f*(x_c + i*phm*y_c)*in (sectoral) or f*z_c*in (axial); in degree L
__device__ void e_mul_linear(const double2 *in, int L, double2 *out, double f,
                             bool axial, double phm, const double *PC,
                             double p) {
  double inv2p = f / (2.0 * p);
  for (int k = 0; k < ntuv(L); ++k) {
    double2 e = in[k];
    if (e.x == 0.0 && e.y == 0.0) continue;
    int t = c_t[k], u = c_u[k], v = c_v[k];
    if (axial) {
      out[k] = cadd(out[k], cscale(e, f * PC[2]));
      int j = hidx(t, u, v + 1);
      out[j] = cadd(out[j], cscale(e, inv2p));
      if (v > 0) {
        j = hidx(t, u, v - 1);
        out[j] = cadd(out[j], cscale(e, f * double(v)));
      }
    } else {
      // (x + i phm y): real factor on x terms, i*phm on y terms
      double2 ie = make_double2(-phm * e.y, phm * e.x);  // i*phm*e
      out[k] = cadd(out[k], cadd(cscale(e, f * PC[0]), cscale(ie, f * PC[1])));
      int j = hidx(t + 1, u, v);
      out[j] = cadd(out[j], cscale(e, inv2p));
      j = hidx(t, u + 1, v);
      out[j] = cadd(out[j], cscale(ie, inv2p));
      if (t > 0) {
        j = hidx(t - 1, u, v);
        out[j] = cadd(out[j], cscale(e, f * double(t)));
      }
      if (u > 0) {
        j = hidx(t, u - 1, v);
        out[j] = cadd(out[j], cscale(ie, f * double(u)));
      }
    }
  }
}

// out += f * r_c^2 * in ; in degree L
__device__ void e_mul_r2(const double2 *in, int L, double2 *out, double f,
                         const double *PC, double PC2, double p) {
  double p2 = 2.0 * p, p22 = p2 * p2;
  for (int k = 0; k < ntuv(L); ++k) {
    double2 e = in[k];
    if (e.x == 0.0 && e.y == 0.0) continue;
    int t = c_t[k], u = c_u[k], v = c_v[k];
    double tt = PC2 + double(2 * (t + u + v) + 3) / p2;
    out[k] = cadd(out[k], cscale(e, f * tt));
    int j;
    j = hidx(t + 2, u, v); out[j] = cadd(out[j], cscale(e, f / p22));
    j = hidx(t, u + 2, v); out[j] = cadd(out[j], cscale(e, f / p22));
    j = hidx(t, u, v + 2); out[j] = cadd(out[j], cscale(e, f / p22));
    j = hidx(t + 1, u, v); out[j] = cadd(out[j], cscale(e, f * PC[0] / p));
    j = hidx(t, u + 1, v); out[j] = cadd(out[j], cscale(e, f * PC[1] / p));
    j = hidx(t, u, v + 1); out[j] = cadd(out[j], cscale(e, f * PC[2] / p));
    if (t > 0) { j = hidx(t - 1, u, v); out[j] = cadd(out[j], cscale(e, f * 2.0 * t * PC[0])); }
    if (u > 0) { j = hidx(t, u - 1, v); out[j] = cadd(out[j], cscale(e, f * 2.0 * u * PC[1])); }
    if (v > 0) { j = hidx(t, u, v - 1); out[j] = cadd(out[j], cscale(e, f * 2.0 * v * PC[2])); }
    if (t > 1) { j = hidx(t - 2, u, v); out[j] = cadd(out[j], cscale(e, f * double(t * (t - 1)))); }
    if (u > 1) { j = hidx(t, u - 2, v); out[j] = cadd(out[j], cscale(e, f * double(u * (u - 1)))); }
    if (v > 1) { j = hidx(t, u, v - 2); out[j] = cadd(out[j], cscale(e, f * double(v * (v - 1)))); }
  }
}

__device__ inline void e_zero(double2 *a, int n) {
  for (int k = 0; k < n; ++k) a[k] = make_double2(0.0, 0.0);
}

// cur (degree L) <- S_{l,m}(r_c) * cur ; returns the new degree
__device__ int e_apply_solid(double2 *cur, double2 *prev, double2 *nx, int L,
                             int l, int m, const double *PC, double PC2,
                             double p) {
  int am = m < 0 ? -m : m;
  double phm = m >= 0 ? 1.0 : -1.0;
  for (int k = 0; k < am; ++k) {
    e_zero(nx, ntuv(L + 1));
    e_mul_linear(cur, L, nx, double(2 * k + 1), false, phm, PC, p);
    for (int i = 0; i < ntuv(L + 1); ++i) cur[i] = nx[i];
    ++L;
  }
  if (l <= am) return L;
  for (int i = 0; i < ntuv(L); ++i) prev[i] = cur[i];
  e_zero(nx, ntuv(L + 1));
  e_mul_linear(cur, L, nx, double(2 * am + 1), true, 0.0, PC, p);
  for (int i = 0; i < ntuv(L + 1); ++i) cur[i] = nx[i];
  ++L;
  for (int ls = am + 1; ls <= l - 1; ++ls) {
    double rlm1 = double(2 * ls + 1) / double(ls - am + 1);
    double rlm2 = -double(ls + am) / double(ls - am + 1);
    e_zero(nx, ntuv(L + 1));
    e_mul_linear(cur, L, nx, rlm1, true, 0.0, PC, p);
    e_mul_r2(prev, L - 1, nx, rlm2, PC, PC2, p);
    for (int i = 0; i < ntuv(L); ++i) prev[i] = cur[i];
    for (int i = 0; i < ntuv(L + 1); ++i) cur[i] = nx[i];
    ++L;
  }
  return L;
}

__device__ double d_fact(int n) {
  double r = 1.0;
  for (int i = 2; i <= n; ++i) r *= double(i);
  return r;
}

// acc += c * [Y*_{l1 m1}(r_A) Y_{l2 m2}(r_B) (r_A^2)^na (r_B^2)^nb] (ESGTF);
// NA: length of the work arrays (>= ntuv of the result degree)
template <int NA>
__device__ void e_esgtf_acc(double2 *acc, double c, int l1, int m1, int l2,
                            int m2, int na, int nb, const Geo &g, double2 *cur,
                            double2 *prev, double2 *nx) {
  if (abs(m1) > l1 || abs(m2) > l2) return;
  e_zero(cur, NA);
  cur[0] = make_double2(g.rkab, 0.0);
  int L = 0;
  L = e_apply_solid(cur, prev, nx, L, l1, -m1, g.PA, g.PA2, g.p);
  L = e_apply_solid(cur, prev, nx, L, l2, m2, g.PB, g.PB2, g.p);
  double phs1 = (m1 > 0 && (m1 & 1)) ? -1.0 : 1.0;
  double phs2 = (m2 > 0 && (m2 & 1)) ? -1.0 : 1.0;
  double dgl = double((2 * l1 + 1) * (2 * l2 + 1));
  double cg1 = d_fact(l1 - abs(m1)) / d_fact(l1 + abs(m1));
  double cg2 = d_fact(l2 - abs(m2)) / d_fact(l2 + abs(m2));
  double ang = phs1 * phs2 * (0.25 / 3.1415926535897932) * sqrt(dgl * cg1 * cg2);
  for (int k = 0; k < ntuv(L); ++k) cur[k] = cscale(cur[k], ang);
  for (int s = 0; s < na; ++s) {
    e_zero(nx, ntuv(L + 2));
    e_mul_r2(cur, L, nx, 1.0, g.PA, g.PA2, g.p);
    L += 2;
    for (int i = 0; i < ntuv(L); ++i) cur[i] = nx[i];
  }
  for (int s = 0; s < nb; ++s) {
    e_zero(nx, ntuv(L + 2));
    e_mul_r2(cur, L, nx, 1.0, g.PB, g.PB2, g.p);
    L += 2;
    for (int i = 0; i < ntuv(L); ++i) cur[i] = nx[i];
  }
  for (int k = 0; k < ntuv(L); ++k) acc[k] = cadd(acc[k], cscale(cur[k], c));
}

__host__ __device__ inline int lval(int k) { return k < 0 ? -k - 1 : k; }

// label index -> (kappa, |m|+1/2) in the order kappa=l (|m| up), kappa=-l-1
__host__ __device__ inline void label_of(int l, int lab, int &kq, int &ma) {
  if (l > 0 && lab < l) {
    kq = l;
    ma = lab + 1;
  } else {
    kq = -l - 1;
    ma = lab - (l > 0 ? l : 0) + 1;
  }
}

__device__ void cg_pair(int kq, int mq, bool small, double &cu, double &cl) {
  int jq = 2 * abs(kq) - 1;
  bool neg = kq < 0;
  if (small) neg = !neg;
  if (neg) {
    cu = sqrt(double(jq + mq) / double(2 * jq));
    cl = sqrt(double(jq - mq) / double(2 * jq));
  } else {
    cu = -sqrt(double(jq - mq + 2) / double(2 * jq + 4));
    cl = sqrt(double(jq + mq + 2) / double(2 * jq + 4));
  }
}

__device__ double rnorm(double ex, int l, bool small) {
  if (!small)
    return exp(0.5 * (log(2.0) - lgamma(l + 1.5) + (l + 1.5) * log(2.0 * ex)));
  return exp(0.5 * (log(2.0) - lgamma(l + 2.5) + (l + 0.5) * log(2.0 * ex)));
}

// One thread per (shell pair, component, label a, label b, set).  Output
// layout per pair and component: [lab_a][lab_b][set][ntuv] complex.
__global__ void k_eqgen(const Shell *sh, int ns, const PairE *pe, int ncomp,
                        double2 *E, long long nwork, const long long *wstart) {
  long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (w >= nwork) return;
  // locate the pair/component by binary search on work starts
  int lo = 0, hi = ns * ns * ncomp - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) / 2;
    if (wstart[mid] <= w) lo = mid; else hi = mid - 1;
  }
  int pc = lo, comp = pc % ncomp, pair = pc / ncomp;
  const Shell &A = sh[pair / ns], &B = sh[pair % ns];
  bool small = comp == 1;
  int nla = 2 * A.l + 1, nlb = 2 * B.l + 1;
  long long r = w - wstart[pc];
  int set = int(r % 2);
  int ib = int((r / 2) % nlb), ia = int(r / 2 / nlb);
  if (ia >= nla) return;
  int ka, ma, kb, mb;
  label_of(A.l, ia, ka, ma);
  label_of(B.l, ib, kb, mb);
  int mqa = (set == 0 ? -1 : 1) * (2 * ma - 1), mqb = -(2 * mb - 1);
  double Ac[3] = {A.x, A.y, A.z}, Bc[3] = {B.x, B.y, B.z};
  Geo g;
  g.p = A.alpha + B.alpha;
  double ab2 = 0.0;
  for (int x = 0; x < 3; ++x) {
    double P = (A.alpha * Ac[x] + B.alpha * Bc[x]) / g.p;
    g.PA[x] = P - Ac[x];
    g.PB[x] = P - Bc[x];
    ab2 += (Ac[x] - Bc[x]) * (Ac[x] - Bc[x]);
  }
  g.PA2 = g.PA[0] * g.PA[0] + g.PA[1] * g.PA[1] + g.PA[2] * g.PA[2];
  g.PB2 = g.PB[0] * g.PB[0] + g.PB[1] * g.PB[1] + g.PB[2] * g.PB[2];
  g.rkab = exp(-(A.alpha * B.alpha * ab2) / g.p);

  double2 acc[NTE], cur[NTE], prev[NTE], nx[NTE];
  e_zero(acc, NTE);
  int la = A.l, lb = B.l;
  double cau, cal, cbu, cbl;
  cg_pair(ka, mqa, small, cau, cal);
  cg_pair(kb, mqb, small, cbu, cbl);
  int l1 = la, l2 = lb;
  double tc[4];
  int tna[4], tnb[4], nterm = 0;
  if (!small) {
    tc[0] = 1.0; tna[0] = 0; tnb[0] = 0; nterm = 1;
  } else {
    l1 = ka < 0 ? la + 1 : la - 1;
    l2 = kb < 0 ? lb + 1 : lb - 1;
    double t22 = 4.0 * A.alpha * B.alpha;
    double t20 = -2.0 * double(2 * lb + 1) * A.alpha;
    double t02 = -2.0 * double(2 * la + 1) * B.alpha;
    double t00 = double((2 * la + 1) * (2 * lb + 1));
    if (ka < 0 && kb < 0) {
      tc[0] = t22; tna[0] = 0; tnb[0] = 0; nterm = 1;
    } else if (ka < 0 && kb > 0) {
      tc[0] = t20; tna[0] = 0; tnb[0] = 0;
      tc[1] = t22; tna[1] = 0; tnb[1] = 1; nterm = 2;
    } else if (ka > 0 && kb < 0) {
      tc[0] = t02; tna[0] = 0; tnb[0] = 0;
      tc[1] = t22; tna[1] = 1; tnb[1] = 0; nterm = 2;
    } else {
      tc[0] = t00; tna[0] = 0; tnb[0] = 0;
      tc[1] = t20; tna[1] = 1; tnb[1] = 0;
      tc[2] = t02; tna[2] = 0; tnb[2] = 1;
      tc[3] = t22; tna[3] = 1; tnb[3] = 1; nterm = 4;
    }
  }
  for (int s = 0; s < 2; ++s) {
    double cab = s == 0 ? cau * cbu : cal * cbl;
    if (fabs(cab) < 1.0e-14) continue;
    int m1 = s == 0 ? (mqa - 1) / 2 : (mqa + 1) / 2;
    int m2 = s == 0 ? (mqb - 1) / 2 : (mqb + 1) / 2;
    for (int t = 0; t < nterm; ++t)
      e_esgtf_acc<NTE>(acc, cab * tc[t], l1, m1, l2, m2, tna[t], tnb[t], g, cur, prev, nx);
  }
  double nrm = rnorm(A.alpha, la, small) * rnorm(B.alpha, lb, small);
  int nt = ntuv(la + lb + (small ? 2 : 0));
  double2 *dst = E + pe[pair].off[comp] + ((long long)(ia * nlb + ib) * 2 + set) * nt;
  for (int k = 0; k < nt; ++k) dst[k] = cscale(acc[k], nrm);
}

// Sparse copy of an E-coefficient block: the nonzero coefficients of each
// (pair, component, label pair, set[, Cartesian component]) block packed to
// the front at the same offset, with their Hermite indices in Eci and the
// sentinel 255 in every slot after the last one.  For pairs on a common axis or centre
// most coefficients vanish by symmetry (exact zeros of the recursion); the
// reference skips them through its E masks (E0LLCD0, BIIFAST IABR11).
constexpr unsigned char ENDIDX = 255;
__global__ void k_ecompact(const double2 *E, double2 *Ecv, unsigned char *Eci, long long nblk,
                           const long long *boff, const int *bnt) {
  long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (b >= nblk) return;
  long long o = boff[b];
  int nt = bnt[b], c = 0;
  for (int k = 0; k < nt; ++k) {
    double2 v = E[o + k];
    if (v.x != 0.0 || v.y != 0.0) {
      Ecv[o + c] = v;
      Eci[o + c] = (unsigned char)k;
      ++c;
    }
  }
  for (int k = c; k < nt; ++k) Eci[o + k] = ENDIDX;  // every slot after the last is a sentinel
}

// ---------------------------------------------------------------------------
// Boys function in the reference's four regimes (FUNFM, bertha-scf.f:32465).
// The power series multiplies by tabulated reciprocals 1/(2n+1) instead of
// dividing (the FP64 pipe is the scarce resource on this part).
// ---------------------------------------------------------------------------
constexpr int NRINV = 2 * (MAXLAM + 2) + 2 * 60 + 4;
__constant__ double c_rinv[NRINV];  // c_rinv[n] = 1/(2n+1)

__device__ void boys_ref(double T, int lam, double *F) {
  const double A0 = 4.994501191201870e-1, B0 = 4.551838436668326e-1;
  const double PI12 = 1.7724538509055160;
  if (T <= 1.0e-11) {
    for (int m = 0; m <= lam; ++m) F[m] = c_rinv[m];
  } else if (T <= 17.0) {
    double txp = exp(-T), tt2 = 2.0 * T, term = 1.0, s = 1.0;
    for (int k = 1; k <= 60; ++k) {
      term = term * tt2 * c_rinv[lam + k];
      s += term;
    }
    F[lam] = s * txp * c_rinv[lam];
    for (int m = lam - 1; m >= 0; --m) F[m] = (tt2 * F[m + 1] + txp) * c_rinv[m];
  } else if (T <= 30.0) {
    double txp = exp(-T), tt2 = 2.0 * T, r2 = 1.0 / tt2;
    F[0] = 0.5 * PI12 / sqrt(T) - txp * (A0 / (B0 + T));
    for (int m = 0; m < lam; ++m) F[m + 1] = (double(2 * m + 1) * F[m] - txp) * r2;
  } else {
    double r2 = 0.5 / T;
    F[0] = 0.5 * PI12 / sqrt(T);
    for (int m = 0; m < lam; ++m) F[m + 1] = double(2 * m + 1) * F[m] * r2;
  }
}

// ---------------------------------------------------------------------------
// Quartet kernel
// ---------------------------------------------------------------------------
struct QArgs {
  const Shell *sh;
  const PairE *pe;
  const double2 *E;
  const double2 *Ecv;        // sparse E values (k_ecompact), same offsets as E
  const unsigned char *Eci;  // their Hermite indices
  const double2 *D;
  double *GD, *GX;
  int ns, ldd, ldf, nskp, isym, racah1;
  int sym;  // 1: also digest the swapped quartet (cd|ab) = (ab|cd) when ab != cd;
            // 2: as 1, lists halved by (ba|dc) = (ab|cd)* (weights, completion)
  double *bound;  // non-null: write max |(ab|cd)| per quartet instead of digesting
  const Inst *inst;  // batched build: per-instance placement (shell .inst), else null
};

constexpr unsigned long long SGN = 0x8000000000000000ULL;

// x * (+-1) through the sign bit, without an FP64 instruction
__device__ inline double flip(double x, unsigned long long m) {
  return __longlong_as_double(__double_as_longlong(x) ^ (long long)m);
}
__device__ inline unsigned long long smask(double p) { return p < 0.0 ? SGN : 0ULL; }

__device__ inline double pair_phase(int kqa, int ma, int kqb, int mb) {
  double s = ((kqa > 0) == (kqb > 0)) ? 1.0 : -1.0;
  return ((ma - mb) & 1) ? -s : s;
}

__device__ inline int ncntrs(int a, int b, int c, int d) {
  int n = 1;
  if (b != a) ++n;
  if (c != a && c != b) ++n;
  if (d != a && d != b && d != c) ++n;
  return n;
}

// CLMFAST label-level selection rules (bertha-scf.f:11843-11939)
__device__ bool label_ok(int isym, int racah1, int mcnt, const int *kq, const int *mq,
                         const int *lq, bool breit = false) {
  int jq[4];
  for (int i = 0; i < 4; ++i) jq[i] = 2 * abs(kq[i]) - 1;
  bool onec = (mcnt == 1 && !racah1);
  if (onec) {
    int nui = max(abs(jq[0] - jq[1]) / 2, abs(jq[2] - jq[3]) / 2);
    int nuf = min((jq[0] + jq[1]) / 2, (jq[2] + jq[3]) / 2);
    if (nui > nuf) return false;
    // a tensor order nu coupling both pairs: both l_a + l_b + nu and
    // l_c + l_d + nu even (CLMFAST :11914-11939); for the Breit
    // interaction also both odd with nu > 0, its magnetic terms (BRTFAST's
    // ISELK, :17443-17456)
    bool selk = false;
    for (int nu = nui; nu <= nuf; ++nu) {
      int pab = (lq[0] + lq[1] + nu) & 1, pcd = (lq[2] + lq[3] + nu) & 1;
      if ((pab == 0 && pcd == 0) || (breit && pab == 1 && pcd == 1 && nu != 0)) selk = true;
    }
    if (!selk) return false;
  }
  if (isym == 1 || isym == 2) {
    bool ok = (mq[0] == mq[1] && mq[2] == mq[3]) || (mq[0] == mq[2] && mq[1] == mq[3]) ||
              (mq[0] == mq[3] && mq[1] == mq[2]);
    if (!ok) return false;
  }
  if (onec) {
    bool selm = false;
    for (int s = 0; s < 16; ++s) {
      int ja = mq[0] * ((s & 8) ? 1 : -1), jb = mq[1] * ((s & 4) ? 1 : -1);
      int jc = mq[2] * ((s & 2) ? 1 : -1), jd = mq[3] * ((s & 1) ? 1 : -1);
      if (ja - jb == jd - jc) selm = true;
    }
    if (!selm) return false;
  }
  return true;
}

__device__ inline double2 ldD(const double2 *D, size_t ld, int i, int j) {
  return D[(size_t)i + ld * j];
}

__device__ inline void satomic(double2 *p, double2 v) {
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}

// FP64 multiply-adds of the two contraction orders of one quartet class:
// ERIFAST's order contracts the ab E-coefficients against R first.
__host__ __device__ inline long long contraction_cost(int pab, int nab, int pcd, int ncd) {
  return 4LL * pab * nab * ncd + 16LL * pab * pcd * ncd;
}

// One CTA per ordered shell quartet.  The pair whose E-coefficients enter
// the first contraction is the "left" pair; it is ab (the reference's order,
// ERIFAST :12676) unless the other order needs fewer multiply-adds, in which
// case (cd|ab) = (ab|cd) is evaluated and the m-sign index is remapped.
__global__ void __launch_bounds__(QT64, 4)
k_quartet(QArgs q, const int4 *quart, long long nq, int t1, int t2) {
  extern __shared__ double smem[];
  double *R = smem;                          // NTR
  double *R2 = R + NTR;                      // NTR
  double *F = R2 + NTR;                      // MAXLAM+2
  double2 *G = (double2 *)(F + MAXLAM + 2);  // CHUNK*2*NTE
  double2 *Jl = G + CHUNK * 2 * NTE;         // MAXSP*MAXSP  J(a,b)
  double2 *Kl = Jl + MAXSP * MAXSP;          // MAXSP*MAXSP  K(a,d)
  double2 *J2 = Kl + MAXSP * MAXSP;          // MAXSP*MAXSP  J(c,d) of (cd|ab)
  double2 *K2 = J2 + MAXSP * MAXSP;          // MAXSP*MAXSP  K(c,b) of (cd|ab)
  __shared__ double sgeo[8];

  for (long long qi = blockIdx.x; qi < nq; qi += gridDim.x) {
    int4 Q4 = quart[qi];
    const Shell &A = q.sh[Q4.x], &B = q.sh[Q4.y], &C = q.sh[Q4.z], &Dd = q.sh[Q4.w];
    int la = A.l, lb = B.l, lc = C.l, ld = Dd.l;
    int degab = la + lb + 2 * t1, degcd = lc + ld + 2 * t2;
    int lam = degab + degcd;
    int nla = 2 * la + 1, nlb = 2 * lb + 1, nlc = 2 * lc + 1, nld = 2 * ld + 1;
    int nlab = nla * nlb, nlcd = nlc * nld;
    int nab = ntuv(degab), ncd = ntuv(degcd);
    bool swp = contraction_cost(nlcd, ncd, nlab, nab) < contraction_cost(nlab, nab, nlcd, ncd);
    int mcnt = ncntrs(A.cnt, B.cnt, C.cnt, Dd.cnt);
    // matrix placement: the call's arrays, or this quartet's instance in a batch
    const double2 *Dm = q.D;
    double *GDm = q.GD, *GXm = q.GX;
    size_t lddm = q.ldd, ldfm = q.ldf;
    int nskpm = q.nskp;
    if (q.inst) {
      const Inst I = q.inst[A.inst];
      if (Dm) Dm += I.off;
      if (GDm) { GDm += 2 * I.off; GXm += 2 * I.off; }
      lddm = ldfm = (size_t)I.ld;
      nskpm = I.nskp;
    }
    if (threadIdx.x == 0) {
      double p = A.alpha + B.alpha, qq = C.alpha + Dd.alpha;
      double Px = (A.alpha * A.x + B.alpha * B.x) / p;
      double Py = (A.alpha * A.y + B.alpha * B.y) / p;
      double Pz = (A.alpha * A.z + B.alpha * B.z) / p;
      double Qx = (C.alpha * C.x + Dd.alpha * Dd.x) / qq;
      double Qy = (C.alpha * C.y + Dd.alpha * Dd.y) / qq;
      double Qz = (C.alpha * C.z + Dd.alpha * Dd.z) / qq;
      double aph = p * qq / (p + qq);
      double T = aph * ((Qx - Px) * (Qx - Px) + (Qy - Py) * (Qy - Py) + (Qz - Pz) * (Qz - Pz));
      boys_ref(T, lam, F);
      // R is built for the left pair's centre minus the right pair's centre
      double sg = swp ? -1.0 : 1.0;
      sgeo[0] = sg * (Px - Qx); sgeo[1] = sg * (Py - Qy); sgeo[2] = sg * (Pz - Qz);
      sgeo[3] = -2.0 * aph;
      sgeo[4] = 2.0 * 17.493418327624863 / (sqrt(p + qq) * p * qq);
      sgeo[6] = 0.0;
    }
    __syncthreads();
    // R recursion: level n = lam..0 ; two buffers
    {
      double X = sgeo[0], Y = sgeo[1], Z = sgeo[2], m2a = sgeo[3];
      double *cur = R, *nxt = R2;
      for (int n = lam; n >= 0; --n) {
        int cnt = ntuv(lam - n);
        for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
          double val;
          if (k == 0) {
            double pw = 1.0;
            for (int i = 0; i < n; ++i) pw *= m2a;
            val = pw * F[n];
          } else {
            int t = c_t[k], u = c_u[k], v = c_v[k];
            if (t > 0) {
              val = X * cur[hidx(t - 1, u, v)];
              if (t > 1) val += double(t - 1) * cur[hidx(t - 2, u, v)];
            } else if (u > 0) {
              val = Y * cur[hidx(t, u - 1, v)];
              if (u > 1) val += double(u - 1) * cur[hidx(t, u - 2, v)];
            } else {
              val = Z * cur[hidx(t, u, v - 1)];
              if (v > 1) val += double(v - 1) * cur[hidx(t, u, v - 2)];
            }
          }
          nxt[k] = val;
        }
        __syncthreads();
        double *tmp = cur; cur = nxt; nxt = tmp;
      }
      double pre = sgeo[4];
      int nt = ntuv(lam);
      if (cur != R)
        for (int k = threadIdx.x; k < nt; k += blockDim.x) R[k] = cur[k] * pre;
      else
        for (int k = threadIdx.x; k < nt; k += blockDim.x) R[k] *= pre;
    }
    for (int k = threadIdx.x; k < MAXSP * MAXSP; k += blockDim.x) {
      Jl[k] = make_double2(0.0, 0.0);
      Kl[k] = make_double2(0.0, 0.0);
      J2[k] = make_double2(0.0, 0.0);
      K2[k] = make_double2(0.0, 0.0);
    }
    bool dual = q.sym && (Q4.x != Q4.z || Q4.y != Q4.w || t1 != t2);
    const double2 *Eab = q.E + q.pe[A.prow + Q4.y].off[t1];
    const double2 *Ecd = q.E + q.pe[C.prow + Q4.w].off[t2];
    // left/right roles
    const double2 *ER = swp ? Eab : Ecd;
    long long oL = swp ? q.pe[C.prow + Q4.w].off[t2] : q.pe[A.prow + Q4.y].off[t1];
    long long oR = swp ? q.pe[A.prow + Q4.y].off[t1] : q.pe[C.prow + Q4.w].off[t2];
    const double2 *ELv = q.Ecv + oL, *ERv = q.Ecv + oR;
    const unsigned char *ELi = q.Eci + oL, *ERi = q.Eci + oR;
    int nL = swp ? ncd : nab, nR = swp ? nab : ncd;
    int nlL = swp ? nlcd : nlab, nlR = swp ? nlab : nlcd;
    int nl2L = swp ? nld : nlb, nl2R = swp ? nlb : nld;  // second label count
    int lq[4] = {la, lb, lc, ld};
    int oab = t1 ? nskpm : 0, ocd = t2 ? nskpm : 0;
    __syncthreads();
    // left labels per pass: as many as the G buffer holds at this degree
    int chunk = max(1, (CHUNK * 2 * NTE) / (2 * nR));
    for (int c0 = 0; c0 < nlL; c0 += chunk) {
      int nch = min(chunk, nlL - c0);
      // first contraction: G[lab][set][q] = Z(q) sum_s E_L[lab][set][s] R[s+q]
      for (int w = threadIdx.x; w < nch * 2 * nR; w += blockDim.x) {
        int lab = w / (2 * nR), rem = w % (2 * nR);
        int set = rem / nR, qq = rem % nR;
        long long eo = ((long long)(c0 + lab) * 2 + set) * nL;
        const double2 *ev_ = ELv + eo;
        const unsigned char *ei = ELi + eo;
        int tq = c_t[qq], uq = c_u[qq], vq = c_v[qq];
        double ax = 0.0, ay = 0.0;
        // nonzero E terms only (sparse copy; see k_ecompact)
        for (int k = 0; k < nL; ++k) {
          int s = ei[k];
          if (s == ENDIDX) break;
          double rv = R[hidx(c_t[s] + tq, c_u[s] + uq, c_v[s] + vq)];
          double2 ev = ev_[k];
          ax = fma(ev.x, rv, ax);
          ay = fma(ev.y, rv, ay);
        }
        unsigned long long zm = ((tq + uq + vq) & 1) ? SGN : 0ULL;
        G[(lab * 2 + set) * nR + qq] = make_double2(flip(ax, zm), flip(ay, zm));
      }
      __syncthreads();
      // second contraction and digestion
      for (int w = threadIdx.x; w < nch * nlR; w += blockDim.x) {
        int lab = w / nlR, lr = w % nlR;
        int labL = c0 + lab;
        int l1 = labL / nl2L, l2 = labL % nl2L, r1 = lr / nl2R, r2 = lr % nl2R;
        int ia = swp ? r1 : l1, ib = swp ? r2 : l2, ic = swp ? l1 : r1, id = swp ? l2 : r2;
        int kq[4], mq[4], mm[4];
        label_of(la, ia, kq[0], mm[0]);
        label_of(lb, ib, kq[1], mm[1]);
        label_of(lc, ic, kq[2], mm[2]);
        label_of(ld, id, kq[3], mm[3]);
        for (int i = 0; i < 4; ++i) mq[i] = 2 * mm[i] - 1;
        if (!label_ok(q.isym, q.racah1, mcnt, kq, mq, lq)) continue;
        double pab = pair_phase(kq[0], mm[0], kq[1], mm[1]);
        double pcd = pair_phase(kq[2], mm[2], kq[3], mm[3]);
        double pl = swp ? pcd : pab, pr = swp ? pab : pcd;
        const double2 *g11 = G + (lab * 2 + 0) * nR, *g21 = G + (lab * 2 + 1) * nR;
        const double2 *e11 = ER + ((long long)lr * 2 + 0) * nR;
        const double2 *e21 = ER + ((long long)lr * 2 + 1) * nR;
        // four complex products (E_R set) x (G set), kept as real partials
        double a0 = 0, b0 = 0, c0r = 0, d0 = 0, a1 = 0, b1 = 0, c1 = 0, d1 = 0;
        double a2 = 0, b2 = 0, c2 = 0, d2 = 0, a3 = 0, b3 = 0, c3 = 0, d3 = 0;
        if (q.isym && !q.bound) {
          // CLMMTZ reads only the real parts of combinations 0, 3, 12, 15
          // (direct) and 0, 6, 9, 15 (exchange): sets 1 and 4 of ERIFAST's
          // linear-molecule path (:12820-12912), 4 of the 16 products, over
          // the nonzero E terms of each set
          long long eo = (long long)lr * 2 * nR;
          const double2 *v1 = ERv + eo, *v2 = v1 + nR;
          const unsigned char *i1 = ERi + eo, *i2 = i1 + nR;
          for (int k = 0; k < nR; ++k) {
            int kk = i1[k];
            if (kk == ENDIDX) break;
            double2 u1 = v1[k], x1 = g11[kk];
            a0 = fma(u1.x, x1.x, a0); b0 = fma(u1.y, x1.y, b0);
          }
          for (int k = 0; k < nR; ++k) {
            int kk = i2[k];
            if (kk == ENDIDX) break;
            double2 u2 = v2[k], x2 = g21[kk];
            a3 = fma(u2.x, x2.x, a3); b3 = fma(u2.y, x2.y, b3);
          }
        } else
        for (int k = 0; k < nR; ++k) {
          double2 u1 = e11[k], u2 = e21[k], x1 = g11[k], x2 = g21[k];
          a0 = fma(u1.x, x1.x, a0); b0 = fma(u1.y, x1.y, b0);
          c0r = fma(u1.x, x1.y, c0r); d0 = fma(u1.y, x1.x, d0);
          a1 = fma(u2.x, x1.x, a1); b1 = fma(u2.y, x1.y, b1);
          c1 = fma(u2.x, x1.y, c1); d1 = fma(u2.y, x1.x, d1);
          a2 = fma(u1.x, x2.x, a2); b2 = fma(u1.y, x2.y, b2);
          c2 = fma(u1.x, x2.y, c2); d2 = fma(u1.y, x2.x, d2);
          a3 = fma(u2.x, x2.x, a3); b3 = fma(u2.y, x2.y, b3);
          c3 = fma(u2.x, x2.y, c3); d3 = fma(u2.y, x2.x, d3);
        }
        // u*x = (a-b, c+d); u*conj(x) = (a+b, d-c)
        double2 s1 = {a0 - b0, c0r + d0}, s1c = {a0 + b0, d0 - c0r};
        double2 s2 = {a1 - b1, c1 + d1}, s2c = {a1 + b1, d1 - c1};
        double2 s3 = {a2 - b2, c2 + d2}, s3c = {a2 + b2, d2 - c2};
        double2 s4 = {a3 - b3, c3 + d3}, s4c = {a3 + b3, d3 - c3};
        // 16 m-sign combinations of (left|right) (ERIFAST :12809-13119);
        // phases are +-1 and applied through the sign bit
        unsigned long long ml = smask(pl), mlr = smask(pl * pr);
        double2 r[16];
        r[0] = s1;
        r[12] = make_double2(flip(s1c.x, ml), flip(s1c.y, ml));
        r[15] = make_double2(flip(r[0].x, mlr), flip(r[0].y, mlr ^ SGN));
        r[3] = make_double2(flip(r[12].x, mlr), flip(r[12].y, mlr ^ SGN));
        r[2] = s2;
        r[14] = make_double2(flip(s2c.x, ml), flip(s2c.y, ml));
        r[13] = make_double2(flip(r[2].x, mlr ^ SGN), flip(r[2].y, mlr));
        r[1] = make_double2(flip(r[14].x, mlr ^ SGN), flip(r[14].y, mlr));
        r[8] = s3;
        r[4] = make_double2(flip(s3c.x, ml ^ SGN), flip(s3c.y, ml ^ SGN));
        r[7] = make_double2(flip(r[8].x, mlr ^ SGN), flip(r[8].y, mlr));
        r[11] = make_double2(flip(r[4].x, mlr ^ SGN), flip(r[4].y, mlr));
        r[10] = s4;
        r[6] = make_double2(flip(s4c.x, ml ^ SGN), flip(s4c.y, ml ^ SGN));
        r[5] = make_double2(flip(r[10].x, mlr), flip(r[10].y, mlr ^ SGN));
        r[9] = make_double2(flip(r[6].x, mlr), flip(r[6].y, mlr ^ SGN));
        // (ab|cd) m-sign index from the (left|right) one
#define RV(sa, sb, sc, sd) (swp ? r[8 * (sc) + 4 * (sd) + 2 * (sa) + (sb)] \
                                : r[8 * (sa) + 4 * (sb) + 2 * (sc) + (sd)])
        int fb[2] = {B.fock[ib][0] + oab, B.fock[ib][1] + oab};
        int fc[2] = {C.fock[ic][0] + ocd, C.fock[ic][1] + ocd};
        int fd[2] = {Dd.fock[id][0] + ocd, Dd.fock[id][1] + ocd};
        if (q.bound) {
          // integral bound mode (Schwarz): largest |(ab|cd)| of the quartet;
          // non-negative doubles order like their bit patterns
          double m = 0.0;
          for (int i = 0; i < 16; ++i) m = fmax(m, fmax(fabs(r[i].x), fabs(r[i].y)));
          atomicMax((unsigned long long *)&sgeo[6], (unsigned long long)__double_as_longlong(m));
          continue;
        }
        if (q.isym == 0) {
          double2 Dcd[4], Dcb[4];
          for (int x = 0; x < 2; ++x)
            for (int y = 0; y < 2; ++y) {
              Dcd[2 * x + y] = ldD(Dm, lddm, fc[x], fd[y]);
              Dcb[2 * x + y] = ldD(Dm, lddm, fc[x], fb[y]);
            }
          for (int sa = 0; sa < 2; ++sa)
            for (int sb = 0; sb < 2; ++sb) {
              double jx = 0.0, jy = 0.0;
              for (int sc = 0; sc < 2; ++sc)
                for (int sd = 0; sd < 2; ++sd) {
                  double2 v = RV(sa, sb, sc, sd), d = Dcd[2 * sc + sd];
                  jx = fma(v.x, d.x, fma(-v.y, d.y, jx));
                  jy = fma(v.x, d.y, fma(v.y, d.x, jy));
                }
              satomic(&Jl[(ia * 2 + sa) * MAXSP + ib * 2 + sb], make_double2(jx, jy));
            }
          for (int sa = 0; sa < 2; ++sa)
            for (int sd = 0; sd < 2; ++sd) {
              double kx = 0.0, ky = 0.0;
              for (int sb = 0; sb < 2; ++sb)
                for (int sc = 0; sc < 2; ++sc) {
                  double2 v = RV(sa, sb, sc, sd), d = Dcb[2 * sc + sb];
                  kx = fma(v.x, d.x, fma(-v.y, d.y, kx));
                  ky = fma(v.x, d.y, fma(v.y, d.x, ky));
                }
              satomic(&Kl[(ia * 2 + sa) * MAXSP + id * 2 + sd], make_double2(kx, ky));
            }
          if (dual) {
            // (cd|ab): J(c,d) += (ab|cd) D(a,b) ; K(c,b) += (ab|cd) D(a,d)
            int fa[2] = {A.fock[ia][0] + oab, A.fock[ia][1] + oab};
            double2 Dab[4], Dad[4];
            for (int x = 0; x < 2; ++x)
              for (int y = 0; y < 2; ++y) {
                Dab[2 * x + y] = ldD(Dm, lddm, fa[x], fb[y]);
                Dad[2 * x + y] = ldD(Dm, lddm, fa[x], fd[y]);
              }
            for (int sc = 0; sc < 2; ++sc)
              for (int sd = 0; sd < 2; ++sd) {
                double jx = 0.0, jy = 0.0;
                for (int sa = 0; sa < 2; ++sa)
                  for (int sb = 0; sb < 2; ++sb) {
                    double2 v = RV(sa, sb, sc, sd), d = Dab[2 * sa + sb];
                    jx = fma(v.x, d.x, fma(-v.y, d.y, jx));
                    jy = fma(v.x, d.y, fma(v.y, d.x, jy));
                  }
                satomic(&J2[(ic * 2 + sc) * MAXSP + id * 2 + sd], make_double2(jx, jy));
              }
            for (int sc = 0; sc < 2; ++sc)
              for (int sb = 0; sb < 2; ++sb) {
                double kx = 0.0, ky = 0.0;
                for (int sa = 0; sa < 2; ++sa)
                  for (int sd = 0; sd < 2; ++sd) {
                    double2 v = RV(sa, sb, sc, sd), d = Dad[2 * sa + sd];
                    kx = fma(v.x, d.x, fma(-v.y, d.y, kx));
                    ky = fma(v.x, d.y, fma(v.y, d.x, ky));
                  }
                satomic(&K2[(ic * 2 + sc) * MAXSP + ib * 2 + sb], make_double2(kx, ky));
              }
          }
        } else {
          // CLMMTZ: real parts, equal-sign direct blocks, crossed exchange
          for (int s = 0; s < 2; ++s) {
            double jv = 0.0, kv = 0.0;
            for (int t = 0; t < 2; ++t) {
              jv = fma(RV(s, s, t, t).x, ldD(Dm, lddm, fc[t], fd[t]).x, jv);
              kv = fma(RV(s, t, t, s).x, ldD(Dm, lddm, fc[t], fb[t]).x, kv);
            }
            atomicAdd(&Jl[(ia * 2 + s) * MAXSP + ib * 2 + s].x, jv);
            atomicAdd(&Kl[(ia * 2 + s) * MAXSP + id * 2 + s].x, kv);
          }
          if (dual) {
            int fa[2] = {A.fock[ia][0] + oab, A.fock[ia][1] + oab};
            for (int s = 0; s < 2; ++s) {
              double jv = 0.0, kv = 0.0;
              for (int t = 0; t < 2; ++t) {
                jv = fma(RV(t, t, s, s).x, ldD(Dm, lddm, fa[t], fb[t]).x, jv);
                kv = fma(RV(t, s, s, t).x, ldD(Dm, lddm, fa[t], fd[t]).x, kv);
              }
              atomicAdd(&J2[(ic * 2 + s) * MAXSP + id * 2 + s].x, jv);
              atomicAdd(&K2[(ic * 2 + s) * MAXSP + ib * 2 + s].x, kv);
            }
          }
        }
#undef RV
      }
      __syncthreads();
    }
    if (q.bound) {
      if (threadIdx.x == 0) q.bound[qi] = sgeo[6];
      __syncthreads();
      continue;
    }
    // weight 1/2 for a quartet equal to its (ba|dc) image, or to its
    // (dc|ba) image within one class: the completion adds it again
    const double wq = (q.sym == 2 && ((Q4.x == Q4.y && Q4.z == Q4.w) ||
                                      (t1 == t2 && Q4.x == Q4.w && Q4.y == Q4.z))) ? 0.5 : 1.0;
    // flush shared accumulators
    {
      int nsa = 2 * nla;
      for (int w = threadIdx.x; w < nsa * 2 * nlb; w += blockDim.x) {
        int a = w / (2 * nlb), b = w % (2 * nlb);
        double2 v = Jl[a * MAXSP + b];
        if (v.x == 0.0 && v.y == 0.0) continue;
        v.x *= wq; v.y *= wq;
        int fa = A.fock[a >> 1][a & 1] + oab, fbb = B.fock[b >> 1][b & 1] + oab;
        double *dst = GDm + 2 * ((size_t)fa + ldfm * fbb);
        atomicAdd(dst, v.x);
        atomicAdd(dst + 1, v.y);
      }
      for (int w = threadIdx.x; w < nsa * 2 * nld; w += blockDim.x) {
        int a = w / (2 * nld), d = w % (2 * nld);
        double2 v = Kl[a * MAXSP + d];
        if (v.x == 0.0 && v.y == 0.0) continue;
        v.x *= wq; v.y *= wq;
        int fa = A.fock[a >> 1][a & 1] + oab, fdd = Dd.fock[d >> 1][d & 1] + ocd;
        double *dst = GXm + 2 * ((size_t)fa + ldfm * fdd);
        atomicAdd(dst, v.x);
        atomicAdd(dst + 1, v.y);
      }
      if (dual) {
        int nsc = 2 * nlc;
        for (int w = threadIdx.x; w < nsc * 2 * nld; w += blockDim.x) {
          int c = w / (2 * nld), d = w % (2 * nld);
          double2 v = J2[c * MAXSP + d];
          if (v.x == 0.0 && v.y == 0.0) continue;
          v.x *= wq; v.y *= wq;
          int fcc = C.fock[c >> 1][c & 1] + ocd, fdd = Dd.fock[d >> 1][d & 1] + ocd;
          double *dst = GDm + 2 * ((size_t)fcc + ldfm * fdd);
          atomicAdd(dst, v.x);
          atomicAdd(dst + 1, v.y);
        }
        for (int w = threadIdx.x; w < nsc * 2 * nlb; w += blockDim.x) {
          int c = w / (2 * nlb), b = w % (2 * nlb);
          double2 v = K2[c * MAXSP + b];
          if (v.x == 0.0 && v.y == 0.0) continue;
          v.x *= wq; v.y *= wq;
          int fcc = C.fock[c >> 1][c & 1] + ocd, fbb = B.fock[b >> 1][b & 1] + oab;
          double *dst = GXm + 2 * ((size_t)fcc + ldfm * fbb);
          atomicAdd(dst, v.x);
          atomicAdd(dst + 1, v.y);
        }
      }
    }
    __syncthreads();
  }
}


// ---------------------------------------------------------------------------
// One-electron matrices (ONEEL bertha-scf.f:6996-7990, OVRLP :6683), FP64.
// ---------------------------------------------------------------------------
constexpr double CLIGHT = 137.035999084;  // speed of light (bertha-scf.f:974)

// Hermite R-integrals R_tuv(alpha, X) for t+u+v <= lam by the same
// recursion as RMAKE, serially in one thread; R and tmp hold NTE values.
__device__ void rints_serial(double X, double Y, double Z, double alpha, int lam,
                             const double *F, double *R, double *tmp) {
  double *cur = R, *nxt = tmp;
  for (int n = lam; n >= 0; --n) {
    int cnt = ntuv(lam - n);
    for (int k = 0; k < cnt; ++k) {
      double val;
      if (k == 0) {
        double pw = 1.0;
        for (int i = 0; i < n; ++i) pw *= -2.0 * alpha;
        val = pw * F[n];
      } else {
        int t = c_t[k], u = c_u[k], v = c_v[k];
        if (t > 0) {
          val = X * cur[hidx(t - 1, u, v)];
          if (t > 1) val += double(t - 1) * cur[hidx(t - 2, u, v)];
        } else if (u > 0) {
          val = Y * cur[hidx(t, u - 1, v)];
          if (u > 1) val += double(u - 1) * cur[hidx(t, u - 2, v)];
        } else {
          val = Z * cur[hidx(t, u, v - 1)];
          if (v > 1) val += double(v - 1) * cur[hidx(t, u, v - 2)];
        }
      }
      nxt[k] = val;
    }
    double *t = cur; cur = nxt; nxt = t;
  }
  if (cur != R)
    for (int k = 0; k < ntuv(lam); ++k) R[k] = cur[k];
}

// -sum_C PNC sum_tuv E_tuv R_tuv(APH, P - C) for the two E sets of one
// label pair: point nuclei (xi = 0) APH = p, PNC = 2 pi Z/p; Gaussian nuclei
// APH = p xi/(p+xi), PNC = 2 pi Z sqrt(xi/(p+xi))/p (ONEEL :7250-7330).
__device__ void nuc_attr2(const double2 *e11, const double2 *e21, int deg, double p,
                          const double *P, const double *nuc, int ncnt, double2 &v11,
                          double2 &v21, double *R, double *tmp) {
  v11 = v21 = make_double2(0.0, 0.0);
  double F[MAXLAM + 2];
  for (int c = 0; c < ncnt; ++c) {
    const double *N = nuc + 5 * c;
    double xi = N[4], aph, pnc;
    if (xi > 0.0) {
      aph = p * xi / (p + xi);
      pnc = 2.0 * 3.1415926535897932 * N[3] * sqrt(xi / (p + xi)) / p;
    } else {
      aph = p;
      pnc = 2.0 * 3.1415926535897932 * N[3] / p;
    }
    double X = P[0] - N[0], Y = P[1] - N[1], Z = P[2] - N[2];
    boys_ref(aph * (X * X + Y * Y + Z * Z), deg, F);
    rints_serial(X, Y, Z, aph, deg, F, R, tmp);
    double a1 = 0.0, b1 = 0.0, a2 = 0.0, b2 = 0.0;
    for (int k = 0; k < ntuv(deg); ++k) {
      a1 = fma(e11[k].x, R[k], a1); b1 = fma(e11[k].y, R[k], b1);
      a2 = fma(e21[k].x, R[k], a2); b2 = fma(e21[k].y, R[k], b2);
    }
    v11.x -= pnc * a1; v11.y -= pnc * b1;
    v21.x -= pnc * a2; v21.y -= pnc * b2;
  }
}

// the four m-sign elements of a one-electron matrix from sets (-|ma|,-|mb|)
// and (+|ma|,-|mb|): (-,+) = -PHS conj(+,-), (+,+) = PHS conj(-,-) (ONEEL
// :7106-7109)
__device__ inline void put4(double2 *M, int ld, const int *r, const int *c, double2 x11,
                           double2 x21, double phs) {
  M[(size_t)r[0] + (size_t)ld * c[0]] = x11;
  M[(size_t)r[1] + (size_t)ld * c[0]] = x21;
  M[(size_t)r[0] + (size_t)ld * c[1]] = make_double2(-phs * x21.x, phs * x21.y);
  M[(size_t)r[1] + (size_t)ld * c[1]] = make_double2(phs * x11.x, -phs * x11.y);
}

// One CTA per ordered shell pair, one thread per label pair: OVLP, HNUC
// (V for LL; V - 2c^2 S for SS) and HKIN (c sqrt((2l+3) alpha) S_SS for the
// LS and SL couplings, or the non-relativistic kinetic matrix for NORL).
// nuc: [ncnt][x, y, z, Z, xi].
__global__ void k_oneel(const Shell *sh, int ns, const PairE *pe, const double2 *E,
                        const double *nuc, int ncnt, int nskp, int norl, double2 *S,
                        double2 *V, double2 *T, int ld) {
  int pair = blockIdx.x;
  const Shell &A = sh[pair / ns], &B = sh[pair % ns];
  int nla = 2 * A.l + 1, nlb = 2 * B.l + 1;
  int lab = threadIdx.x;
  if (lab >= nla * nlb) return;
  int ia = lab / nlb, ib = lab % nlb;
  int ka, ma, kb, mb;
  label_of(A.l, ia, ka, ma);
  label_of(B.l, ib, kb, mb);
  double phs = pair_phase(ka, ma, kb, mb);
  double p = A.alpha + B.alpha;
  double P[3] = {(A.alpha * A.x + B.alpha * B.x) / p, (A.alpha * A.y + B.alpha * B.y) / p,
                 (A.alpha * A.z + B.alpha * B.z) / p};
  double eroot = pow(3.1415926535897932 / p, 1.5);
  int r[2] = {A.fock[ia][0], A.fock[ia][1]}, c[2] = {B.fock[ib][0], B.fock[ib][1]};
  double R[NTE], tmp[NTE];
  // LL
  int degl = A.l + B.l, ntl = ntuv(degl);
  const double2 *l11 = E + pe[pair].off[0] + (long long)(lab * 2 + 0) * ntl;
  const double2 *l21 = l11 + ntl;
  put4(S, ld, r, c, cscale(l11[0], eroot), cscale(l21[0], eroot), phs);
  double2 v11, v21;
  nuc_attr2(l11, l21, degl, p, P, nuc, ncnt, v11, v21, R, tmp);
  put4(V, ld, r, c, v11, v21, phs);
  if (norl) {
    double PB[3] = {P[0] - B.x, P[1] - B.y, P[2] - B.z};
    double pb2 = PB[0] * PB[0] + PB[1] * PB[1] + PB[2] * PB[2], eb = B.alpha;
    double e0 = eb * (2 * B.l + 3) - 2.0 * eb * eb * pb2 - 3.0 * eb * eb / p, e1 = 4.0 * eb * eb;
    double2 t[2];
    const double2 *ee[2] = {l11, l21};
    for (int s2 = 0; s2 < 2; ++s2) {
      const double2 *e = ee[s2];
      double2 tr = cscale(e[0], e0);
      if (degl >= 1) {
        double2 d = cadd(cadd(cscale(e[hidx(1, 0, 0)], PB[0]), cscale(e[hidx(0, 1, 0)], PB[1])),
                         cscale(e[hidx(0, 0, 1)], PB[2]));
        tr = cadd(tr, cscale(d, -e1));
      }
      if (degl >= 2) {
        double2 d = cadd(cadd(e[hidx(2, 0, 0)], e[hidx(0, 2, 0)]), e[hidx(0, 0, 2)]);
        tr = cadd(tr, cscale(d, -e1));
      }
      t[s2] = cscale(tr, eroot);
    }
    put4(T, ld, r, c, t[0], t[1], phs);
    return;
  }
  // SS
  int degs = degl + 2, nts = ntuv(degs);
  const double2 *s11 = E + pe[pair].off[1] + (long long)(lab * 2 + 0) * nts;
  const double2 *s21 = s11 + nts;
  int rs[2] = {r[0] + nskp, r[1] + nskp}, cs[2] = {c[0] + nskp, c[1] + nskp};
  double2 ss11 = cscale(s11[0], eroot), ss21 = cscale(s21[0], eroot);
  put4(S, ld, rs, cs, ss11, ss21, phs);
  nuc_attr2(s11, s21, degs, p, P, nuc, ncnt, v11, v21, R, tmp);
  double cv2 = 2.0 * CLIGHT * CLIGHT;
  put4(V, ld, rs, cs, cadd(v11, cscale(ss11, -cv2)), cadd(v21, cscale(ss21, -cv2)), phs);
  double fsl = CLIGHT * sqrt((2 * B.l + 3) * B.alpha);  // T(a_S, b_L)
  double fls = CLIGHT * sqrt((2 * A.l + 3) * A.alpha);  // T(a_L, b_S)
  put4(T, ld, rs, c, cscale(ss11, fsl), cscale(ss21, fsl), phs);
  put4(T, ld, r, cs, cscale(ss11, fls), cscale(ss21, fls), phs);
}

// ---------------------------------------------------------------------------
// Breit / Gaunt interaction (BRTFAST :17060, BIIFAST :18337, BRTMTG :19815,
// BRTMTZ :19172), FP64.
// ---------------------------------------------------------------------------
constexpr int NTB = ntuv(2 * MAXLB + 1);  // E terms of an LS/SL pair (120)
constexpr int NTW = ntuv(4 * MAXLB + 2);  // Breit kernel entries per quartet (680)
constexpr int BCHUNK = 1;                 // ab labels per pass at the largest cd degree

// sigma-coupled E-coefficients psi_a^+ sigma_q psi_b, q = x, y, z, for the
// component pairs LS (comp 0: a large, b small, times i; EQLS :34937) and SL
// (comp 1: a small, b large, times -i; EQSL :35433), sigma_y carrying the
// extra factor i of both.  One thread per (pair, comp, lab_a, lab_b, set, q);
// layout per pair and comp: [lab_a][lab_b][set][q][ntuv(la+lb+1)].
__global__ void k_eqgen_q(const Shell *sh, int ns, const long long *offq, double2 *E,
                          long long nwork, const long long *wstart) {
  long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (w >= nwork) return;
  int lo = 0, hi = ns * ns * 2 - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) / 2;
    if (wstart[mid] <= w) lo = mid; else hi = mid - 1;
  }
  int pc = lo, comp = pc % 2, pair = pc / 2;
  const Shell &A = sh[pair / ns], &B = sh[pair % ns];
  int nlb = 2 * B.l + 1;
  long long r = w - wstart[pc];
  int q = int(r % 3);
  int set = int((r / 3) % 2);
  int ib = int((r / 6) % nlb), ia = int(r / 6 / nlb);
  if (ia >= 2 * A.l + 1) return;
  int ka, ma, kb, mb;
  label_of(A.l, ia, ka, ma);
  label_of(B.l, ib, kb, mb);
  int mqa = (set == 0 ? -1 : 1) * (2 * ma - 1), mqb = -(2 * mb - 1);
  double Ac[3] = {A.x, A.y, A.z}, Bc[3] = {B.x, B.y, B.z};
  Geo g;
  g.p = A.alpha + B.alpha;
  double ab2 = 0.0;
  for (int x = 0; x < 3; ++x) {
    double P = (A.alpha * Ac[x] + B.alpha * Bc[x]) / g.p;
    g.PA[x] = P - Ac[x];
    g.PB[x] = P - Bc[x];
    ab2 += (Ac[x] - Bc[x]) * (Ac[x] - Bc[x]);
  }
  g.PA2 = g.PA[0] * g.PA[0] + g.PA[1] * g.PA[1] + g.PA[2] * g.PA[2];
  g.PB2 = g.PB[0] * g.PB[0] + g.PB[1] * g.PB[1] + g.PB[2] * g.PB[2];
  g.rkab = exp(-(A.alpha * B.alpha * ab2) / g.p);
  bool sa = comp == 1, sb = comp == 0;
  double cau, cal, cbu, cbl;
  cg_pair(ka, mqa, sa, cau, cal);
  cg_pair(kb, mqb, sb, cbu, cbl);
  // radial terms (coefficient, power of r^2) of each component
  double ca[2], cb[2];
  int na[2], nb[2], nta, ntb, l1, l2;
  if (!sa) { l1 = A.l; ca[0] = 1.0; na[0] = 0; nta = 1; }
  else if (ka < 0) { l1 = A.l + 1; ca[0] = -2.0 * A.alpha; na[0] = 0; nta = 1; }
  else { l1 = A.l - 1; ca[0] = double(2 * A.l + 1); na[0] = 0; ca[1] = -2.0 * A.alpha; na[1] = 1; nta = 2; }
  if (!sb) { l2 = B.l; cb[0] = 1.0; nb[0] = 0; ntb = 1; }
  else if (kb < 0) { l2 = B.l + 1; cb[0] = -2.0 * B.alpha; nb[0] = 0; ntb = 1; }
  else { l2 = B.l - 1; cb[0] = double(2 * B.l + 1); nb[0] = 0; cb[1] = -2.0 * B.alpha; nb[1] = 1; ntb = 2; }
  // spin terms: (upper/lower of a, upper/lower of b, weight)
  int ua[2], ub[2];
  double wt[2];
  if (q == 0) { ua[0] = 0; ub[0] = 1; wt[0] = 1.0; ua[1] = 1; ub[1] = 0; wt[1] = 1.0; }
  else if (q == 1) { ua[0] = 0; ub[0] = 1; wt[0] = -1.0; ua[1] = 1; ub[1] = 0; wt[1] = 1.0; }
  else { ua[0] = 0; ub[0] = 0; wt[0] = 1.0; ua[1] = 1; ub[1] = 1; wt[1] = -1.0; }
  double2 acc[NTB], cur[NTB], prev[NTB], nx[NTB];
  e_zero(acc, NTB);
  for (int st = 0; st < 2; ++st) {
    double cab = (ua[st] == 0 ? cau : cal) * (ub[st] == 0 ? cbu : cbl);
    if (fabs(cab) < 1.0e-14) continue;
    int m1 = ua[st] == 0 ? (mqa - 1) / 2 : (mqa + 1) / 2;
    int m2 = ub[st] == 0 ? (mqb - 1) / 2 : (mqb + 1) / 2;
    for (int i = 0; i < nta; ++i)
      for (int j = 0; j < ntb; ++j)
        e_esgtf_acc<NTB>(acc, wt[st] * cab * ca[i] * cb[j], l1, m1, l2, m2, na[i], nb[j], g,
                         cur, prev, nx);
  }
  double nrm = rnorm(A.alpha, A.l, sa) * rnorm(B.alpha, B.l, sb);
  // i (LS) or -i (SL), times i again for sigma_y
  double ph = sa ? -1.0 : 1.0;
  int nt = ntuv(A.l + B.l + 1);
  double2 *dst = E + offq[(size_t)pair * 2 + comp] + (((long long)(ia * nlb + ib) * 2 + set) * 3 + q) * nt;
  for (int k = 0; k < nt; ++k) {
    double2 v = cscale(acc[k], nrm * ph);
    dst[k] = q == 1 ? make_double2(-v.x, -v.y) : make_double2(-v.y, v.x);
  }
}

struct BArgs {
  const Shell *sh;
  const long long *offq;
  const double2 *E;
  const double2 *Ecv;        // sparse E values (k_ecompact), same offsets as E
  const unsigned char *Eci;  // their Hermite indices
  const double2 *D;
  double *BX;
  int ns, ldd, ldf, nskp, isym, racah1, gaunt;
  int dual;  // also digest (cd|ab) = (ab|cd): K(c,b) += (ab|cd) D(a,d); 2: the
             // (LS|SL) list is also halved by (dc|ba) = (ab|cd)* (weights)
  double *bound;  // non-null: write max |(ab|cd)| per quartet instead of digesting
};

__device__ inline double2 ldDB(const BArgs &q, int i, int j) {
  return q.D[(size_t)i + (size_t)q.ldd * j];
}

// The Breit kernel table is symmetric, W_ij(N) = W_ji(N) (the operator's
// Cartesian part delta_ij/r + r_i r_j/r^3 is), so 6 entries per N are kept:
// xx, yy, zz, xy, xz, yz.
__host__ __device__ inline int sym6(int i, int j) { return i == j ? i : i + j + 2; }

// doubles of the region after the table: the first contraction's G buffer,
// which the two R recursion buffers alias
constexpr int BREG = (BCHUNK * 2 * 3 * NTB * 2 > 2 * NTR) ? BCHUNK * 2 * 3 * NTB * 2 : 2 * NTR;

size_t breit_smem() {
  return sizeof(double) * (NTW * 6 + BREG) + sizeof(double2) * (2 * MAXSP * MAXSP);
}

// FP64 multiply-adds of the two contraction orders of a Breit quartet: the
// left pair's E against the 3x3 kernel (3 components of each electron, 1
// for the Gaunt term alone), then the second contraction over 3 components
// with 16 products (4 when only the real digestion's are needed).
__host__ __device__ inline long long breit_cost(int pl, int nl, int pr, int nr, int gaunt,
                                                bool lin) {
  return 2LL * pl * nl * nr * (gaunt ? 3 : 9) + 3LL * (lin ? 4 : 16) * pl * pr * nr;
}

// One CTA per shell quartet of component class (t1|t2), t = 0 LS, 1 SL.
// R-integrals to order degab+degcd+2, the 3x3 Breit kernel table
//   W_ij(N) = BFAC (delta_ij R_N - T_ij(N)),
//   T_ij(N) = R_{N+e_i+e_j}/(2 alpha) - R_{N+e_i} PQ_j + N_j R_{N+e_i-e_j}
// (BIIFAST :18655-18880; Gaunt: W_ij = -delta_ij R_N), the first contraction
// G_i = sum_j E_j(ab) W_ij for both E sets, the second contraction summed
// over i, the 16 m-sign combinations with the Breit phases (Coulomb phases
// negated, :17528-17533 and :18899) and the exchange digestion of BRTMTG/BRTMTZ batch type 5.
__global__ void __launch_bounds__(QT64, 4)
k_breit(BArgs q, const int4 *quart, long long nq, int t1, int t2) {
  extern __shared__ double smem[];
  double *W = smem;                          // NTW*6 (symmetric table)
  double2 *G = (double2 *)(W + NTW * 6);     // BCHUNK*2*3*NTB
  double *R = (double *)G;                   // R recursion scratch (aliases G)
  double *R2 = R + NTR;
  double2 *Kl = (double2 *)((double *)G + BREG);  // MAXSP*MAXSP  K(a,d)
  double2 *K2 = Kl + MAXSP * MAXSP;          // MAXSP*MAXSP  K(c,b) of (cd|ab)
  __shared__ double sgeo[10];
  __shared__ double F[MAXLAM + 2];
  for (long long qi = blockIdx.x; qi < nq; qi += gridDim.x) {
    int4 Q4 = quart[qi];
    const Shell &A = q.sh[Q4.x], &B = q.sh[Q4.y], &C = q.sh[Q4.z], &Dd = q.sh[Q4.w];
    int la = A.l, lb = B.l, lc = C.l, ld = Dd.l;
    int degab = la + lb + 1, degcd = lc + ld + 1;
    int lamn = degab + degcd, lam = lamn + (q.gaunt ? 0 : 2);
    int nla = 2 * la + 1, nlb = 2 * lb + 1, nlc = 2 * lc + 1, nld = 2 * ld + 1;
    int nlab = nla * nlb, nlcd = nlc * nld;
    int nab = ntuv(degab), ncd = ntuv(degcd);
    int mcnt = ncntrs(A.cnt, B.cnt, C.cnt, Dd.cnt);
    bool dual = q.dual && (Q4.x != Q4.z || Q4.y != Q4.w || t1 != t2);
    bool lin = q.isym && !q.bound;  // only the 4 products of the real digestion
    bool swp = breit_cost(nlcd, ncd, nlab, nab, q.gaunt, lin) <
               breit_cost(nlab, nab, nlcd, ncd, q.gaunt, lin);
    if (threadIdx.x == 0) {
      double p = A.alpha + B.alpha, qq = C.alpha + Dd.alpha;
      double Px = (A.alpha * A.x + B.alpha * B.x) / p;
      double Py = (A.alpha * A.y + B.alpha * B.y) / p;
      double Pz = (A.alpha * A.z + B.alpha * B.z) / p;
      double Qx = (C.alpha * C.x + Dd.alpha * Dd.x) / qq;
      double Qy = (C.alpha * C.y + Dd.alpha * Dd.y) / qq;
      double Qz = (C.alpha * C.z + Dd.alpha * Dd.z) / qq;
      double aph = p * qq / (p + qq);
      double T = aph * ((Qx - Px) * (Qx - Px) + (Qy - Py) * (Qy - Py) + (Qz - Pz) * (Qz - Pz));
      boys_ref(T, lam, F);
      // R and the kernel table are built for the left pair's centre minus
      // the right pair's: the Breit kernel is even in P - Q, so swapping the
      // pairs only flips the sign of odd Hermite orders
      double sg = swp ? -1.0 : 1.0;
      sgeo[0] = sg * (Px - Qx); sgeo[1] = sg * (Py - Qy); sgeo[2] = sg * (Pz - Qz);
      sgeo[3] = -2.0 * aph;
      sgeo[4] = 2.0 * 17.493418327624863 / (sqrt(p + qq) * p * qq);
      sgeo[5] = 0.5 / aph;
      sgeo[6] = sg * (Qx - Px); sgeo[7] = sg * (Qy - Py); sgeo[8] = sg * (Qz - Pz);
      sgeo[9] = 0.0;
    }
    __syncthreads();
    {
      double X = sgeo[0], Y = sgeo[1], Z = sgeo[2], m2a = sgeo[3];
      double *cur = R, *nxt = R2;
      for (int n = lam; n >= 0; --n) {
        int cnt = ntuv(lam - n);
        for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
          double val;
          if (k == 0) {
            double pw = 1.0;
            for (int i = 0; i < n; ++i) pw *= m2a;
            val = pw * F[n];
          } else {
            int t = c_t[k], u = c_u[k], v = c_v[k];
            if (t > 0) {
              val = X * cur[hidx(t - 1, u, v)];
              if (t > 1) val += double(t - 1) * cur[hidx(t - 2, u, v)];
            } else if (u > 0) {
              val = Y * cur[hidx(t, u - 1, v)];
              if (u > 1) val += double(u - 1) * cur[hidx(t, u - 2, v)];
            } else {
              val = Z * cur[hidx(t, u, v - 1)];
              if (v > 1) val += double(v - 1) * cur[hidx(t, u, v - 2)];
            }
          }
          nxt[k] = val;
        }
        __syncthreads();
        double *tmp = cur; cur = nxt; nxt = tmp;
      }
      // kernel table from PRE*R (cur holds R)
      double pre = sgeo[4], h2a = sgeo[5];
      double pq[3] = {sgeo[6], sgeo[7], sgeo[8]};
      double bfac = q.gaunt ? -1.0 : -0.5;
      int nw = ntuv(lamn);
      for (int w = threadIdx.x; w < nw * 6; w += blockDim.x) {
        int n = w / 6, e = w % 6;
        int i = e < 3 ? e : (e == 5 ? 1 : 0), j = e < 3 ? e : (e == 3 ? 1 : 2);
        int N[3] = {c_t[n], c_u[n], c_v[n]};
        double rn = cur[n] * pre;
        double val;
        if (q.gaunt) {
          val = i == j ? -rn : 0.0;
        } else {
          int a[3] = {N[0], N[1], N[2]};
          a[i] += 1;
          a[j] += 1;
          double tt = cur[hidx(a[0], a[1], a[2])] * h2a;
          a[j] -= 1;
          tt -= cur[hidx(a[0], a[1], a[2])] * pq[j];
          a[j] -= 1;
          if (a[j] >= 0) tt += cur[hidx(a[0], a[1], a[2])] * double(N[j]);
          val = bfac * ((i == j ? rn : 0.0) - tt * pre);
        }
        W[w] = val;
      }
    }
    for (int k = threadIdx.x; k < MAXSP * MAXSP; k += blockDim.x) {
      Kl[k] = make_double2(0.0, 0.0);
      K2[k] = make_double2(0.0, 0.0);
    }
    __syncthreads();
    const double2 *Eab = q.E + q.offq[((size_t)Q4.x * q.ns + Q4.y) * 2 + t1];
    const double2 *Ecd = q.E + q.offq[((size_t)Q4.z * q.ns + Q4.w) * 2 + t2];
    // left/right roles
    const double2 *ER = swp ? Eab : Ecd;
    long long oL = q.offq[swp ? ((size_t)Q4.z * q.ns + Q4.w) * 2 + t2 : ((size_t)Q4.x * q.ns + Q4.y) * 2 + t1];
    long long oR = q.offq[swp ? ((size_t)Q4.x * q.ns + Q4.y) * 2 + t1 : ((size_t)Q4.z * q.ns + Q4.w) * 2 + t2];
    const double2 *ELv = q.Ecv + oL, *ERv = q.Ecv + oR;
    const unsigned char *ELi = q.Eci + oL, *ERi = q.Eci + oR;
    int nL = swp ? ncd : nab, nR = swp ? nab : ncd;
    int nlL = swp ? nlcd : nlab, nlR = swp ? nlab : nlcd;
    int nl2L = swp ? nld : nlb, nl2R = swp ? nlb : nld;
    int lq[4] = {la, lb, lc, ld};
    // Fock offsets: an LS pair has its first function large, second small
    int oa = t1 ? q.nskp : 0, ob = t1 ? 0 : q.nskp;
    int oc = t2 ? q.nskp : 0, od = t2 ? 0 : q.nskp;
    // as many ab labels per pass as the G buffer holds (fewer barriers and
    // idle threads for low angular momenta)
    int chunk = max(1, (BCHUNK * 2 * 3 * NTB) / (6 * nR));
    for (int c0 = 0; c0 < nlL; c0 += chunk) {
      int nch = min(chunk, nlL - c0);
      // first contraction: G[lab][set][i][q] = Z(q) sum_j sum_s E_j[s] W_ij(s+q)
      for (int w = threadIdx.x; w < nch * 6 * nR; w += blockDim.x) {
        int lab = w / (6 * nR), rem = w % (6 * nR);
        int set = rem / (3 * nR), i = (rem / nR) % 3, qq = rem % nR;
        long long eo = ((long long)(c0 + lab) * 2 + set) * 3 * nL;
        int tq = c_t[qq], uq = c_u[qq], vq = c_v[qq];
        double ax = 0.0, ay = 0.0;
        // nonzero E terms of each Cartesian component j (sparse copy)
        for (int j = 0; j < 3; ++j) {
          const double2 *ev_ = ELv + eo + j * nL;
          const unsigned char *ei = ELi + eo + j * nL;
          for (int k = 0; k < nL; ++k) {
            int s = ei[k];
            if (s == ENDIDX) break;
            double w = W[hidx(c_t[s] + tq, c_u[s] + uq, c_v[s] + vq) * 6 + sym6(i, j)];
            double2 ev = ev_[k];
            ax = fma(ev.x, w, ax);
            ay = fma(ev.y, w, ay);
          }
        }
        unsigned long long zm = ((tq + uq + vq) & 1) ? SGN : 0ULL;
        G[((lab * 2 + set) * 3 + i) * nR + qq] = make_double2(flip(ax, zm), flip(ay, zm));
      }
      __syncthreads();
      // second contraction and exchange digestion
      for (int w = threadIdx.x; w < nch * nlR; w += blockDim.x) {
        int lab = w / nlR, lr = w % nlR;
        int labL = c0 + lab;
        int l1 = labL / nl2L, l2 = labL % nl2L, r1 = lr / nl2R, r2 = lr % nl2R;
        int ia = swp ? r1 : l1, ib = swp ? r2 : l2, ic = swp ? l1 : r1, id = swp ? l2 : r2;
        int kq[4], mq[4], mm[4];
        label_of(la, ia, kq[0], mm[0]);
        label_of(lb, ib, kq[1], mm[1]);
        label_of(lc, ic, kq[2], mm[2]);
        label_of(ld, id, kq[3], mm[3]);
        for (int i = 0; i < 4; ++i) mq[i] = 2 * mm[i] - 1;
        if (!label_ok(q.isym, q.racah1, mcnt, kq, mq, lq, true)) continue;
        double pab = -pair_phase(kq[0], mm[0], kq[1], mm[1]);
        double pcd = -pair_phase(kq[2], mm[2], kq[3], mm[3]);
        double pl = swp ? pcd : pab, pr = swp ? pab : pcd;
        double a0 = 0, b0 = 0, c0r = 0, d0 = 0, a1 = 0, b1 = 0, c1 = 0, d1 = 0;
        double a2 = 0, b2 = 0, c2 = 0, d2 = 0, a3 = 0, b3 = 0, c3 = 0, d3 = 0;
        for (int i = 0; i < 3; ++i) {
          const double2 *g11 = G + ((lab * 2 + 0) * 3 + i) * nR;
          const double2 *g21 = G + ((lab * 2 + 1) * 3 + i) * nR;
          const double2 *e11 = ER + (((long long)lr * 2 + 0) * 3 + i) * nR;
          const double2 *e21 = ER + (((long long)lr * 2 + 1) * 3 + i) * nR;
          if (lin) {
            // BRTMTZ reads only the real parts of combinations 0, 6, 9, 15;
            // nonzero E terms of each set only
            long long e1o = (((long long)lr * 2 + 0) * 3 + i) * nR;
            long long e2o = (((long long)lr * 2 + 1) * 3 + i) * nR;
            for (int k = 0; k < nR; ++k) {
              int kk = ERi[e1o + k];
              if (kk == ENDIDX) break;
              double2 u1 = ERv[e1o + k], x1 = g11[kk];
              a0 = fma(u1.x, x1.x, a0); b0 = fma(u1.y, x1.y, b0);
            }
            for (int k = 0; k < nR; ++k) {
              int kk = ERi[e2o + k];
              if (kk == ENDIDX) break;
              double2 u2 = ERv[e2o + k], x2 = g21[kk];
              a3 = fma(u2.x, x2.x, a3); b3 = fma(u2.y, x2.y, b3);
            }
            continue;
          }
          for (int k = 0; k < nR; ++k) {
            double2 u1 = e11[k], u2 = e21[k], x1 = g11[k], x2 = g21[k];
            a0 = fma(u1.x, x1.x, a0); b0 = fma(u1.y, x1.y, b0);
            c0r = fma(u1.x, x1.y, c0r); d0 = fma(u1.y, x1.x, d0);
            a1 = fma(u2.x, x1.x, a1); b1 = fma(u2.y, x1.y, b1);
            c1 = fma(u2.x, x1.y, c1); d1 = fma(u2.y, x1.x, d1);
            a2 = fma(u1.x, x2.x, a2); b2 = fma(u1.y, x2.y, b2);
            c2 = fma(u1.x, x2.y, c2); d2 = fma(u1.y, x2.x, d2);
            a3 = fma(u2.x, x2.x, a3); b3 = fma(u2.y, x2.y, b3);
            c3 = fma(u2.x, x2.y, c3); d3 = fma(u2.y, x2.x, d3);
          }
        }
        double2 s1 = {a0 - b0, c0r + d0}, s1c = {a0 + b0, d0 - c0r};
        double2 s2 = {a1 - b1, c1 + d1}, s2c = {a1 + b1, d1 - c1};
        double2 s3 = {a2 - b2, c2 + d2}, s3c = {a2 + b2, d2 - c2};
        double2 s4 = {a3 - b3, c3 + d3}, s4c = {a3 + b3, d3 - c3};
        unsigned long long ml = smask(pl), mlr = smask(pl * pr);
        double2 r[16];
        r[0] = s1;
        r[12] = make_double2(flip(s1c.x, ml), flip(s1c.y, ml));
        r[15] = make_double2(flip(r[0].x, mlr), flip(r[0].y, mlr ^ SGN));
        r[3] = make_double2(flip(r[12].x, mlr), flip(r[12].y, mlr ^ SGN));
        r[2] = s2;
        r[14] = make_double2(flip(s2c.x, ml), flip(s2c.y, ml));
        r[13] = make_double2(flip(r[2].x, mlr ^ SGN), flip(r[2].y, mlr));
        r[1] = make_double2(flip(r[14].x, mlr ^ SGN), flip(r[14].y, mlr));
        r[8] = s3;
        r[4] = make_double2(flip(s3c.x, ml ^ SGN), flip(s3c.y, ml ^ SGN));
        r[7] = make_double2(flip(r[8].x, mlr ^ SGN), flip(r[8].y, mlr));
        r[11] = make_double2(flip(r[4].x, mlr ^ SGN), flip(r[4].y, mlr));
        r[10] = s4;
        r[6] = make_double2(flip(s4c.x, ml ^ SGN), flip(s4c.y, ml ^ SGN));
        r[5] = make_double2(flip(r[10].x, mlr), flip(r[10].y, mlr ^ SGN));
        r[9] = make_double2(flip(r[6].x, mlr), flip(r[6].y, mlr ^ SGN));
        if (q.bound) {
          // bound mode (Schwarz): largest |(ab|cd)| of the quartet
          double m = 0.0;
          for (int i = 0; i < 16; ++i) m = fmax(m, fmax(fabs(r[i].x), fabs(r[i].y)));
          atomicMax((unsigned long long *)&sgeo[9], (unsigned long long)__double_as_longlong(m));
          continue;
        }
        // (ab|cd) m-sign index from the (left|right) one
#define RB(sa, sb, sc, sd) (swp ? r[8 * (sc) + 4 * (sd) + 2 * (sa) + (sb)] \
                                : r[8 * (sa) + 4 * (sb) + 2 * (sc) + (sd)])
        int fa[2] = {A.fock[ia][0] + oa, A.fock[ia][1] + oa};
        int fb[2] = {B.fock[ib][0] + ob, B.fock[ib][1] + ob};
        int fc[2] = {C.fock[ic][0] + oc, C.fock[ic][1] + oc};
        int fd[2] = {Dd.fock[id][0] + od, Dd.fock[id][1] + od};
        if (q.isym == 0) {
          for (int sa = 0; sa < 2; ++sa)
            for (int sd = 0; sd < 2; ++sd) {
              double kx = 0.0, ky = 0.0;
              for (int sb = 0; sb < 2; ++sb)
                for (int sc = 0; sc < 2; ++sc) {
                  double2 v = RB(sa, sb, sc, sd), d = ldDB(q, fc[sc], fb[sb]);
                  kx = fma(v.x, d.x, fma(-v.y, d.y, kx));
                  ky = fma(v.x, d.y, fma(v.y, d.x, ky));
                }
              satomic(&Kl[(ia * 2 + sa) * MAXSP + id * 2 + sd], make_double2(kx, ky));
            }
          if (dual)
            for (int sc = 0; sc < 2; ++sc)
              for (int sb = 0; sb < 2; ++sb) {
                double kx = 0.0, ky = 0.0;
                for (int sa = 0; sa < 2; ++sa)
                  for (int sd = 0; sd < 2; ++sd) {
                    double2 v = RB(sa, sb, sc, sd), d = ldDB(q, fa[sa], fd[sd]);
                    kx = fma(v.x, d.x, fma(-v.y, d.y, kx));
                    ky = fma(v.x, d.y, fma(v.y, d.x, ky));
                  }
                satomic(&K2[(ic * 2 + sc) * MAXSP + ib * 2 + sb], make_double2(kx, ky));
              }
        } else {
          // BRTMTZ: real parts, crossed exchange blocks
          for (int s = 0; s < 2; ++s) {
            double kv = 0.0;
            for (int t = 0; t < 2; ++t)
              kv = fma(RB(s, t, t, s).x, ldDB(q, fc[t], fb[t]).x, kv);
            atomicAdd(&Kl[(ia * 2 + s) * MAXSP + id * 2 + s].x, kv);
          }
          if (dual)
            for (int s = 0; s < 2; ++s) {
              double kv = 0.0;
              for (int t = 0; t < 2; ++t)
                kv = fma(RB(t, s, s, t).x, ldDB(q, fa[t], fd[t]).x, kv);
              atomicAdd(&K2[(ic * 2 + s) * MAXSP + ib * 2 + s].x, kv);
            }
        }
#undef RB
      }
      __syncthreads();
    }
    if (q.bound) {
      if (threadIdx.x == 0) q.bound[qi] = sgeo[9];
      __syncthreads();
      continue;
    }
    // flush shared accumulators; in a halved (LS|SL) list a quartet equal
    // to its (dc|ba) image counts 1/2 (the completion adds it again)
    const double wq = (q.dual == 2 && t2 == 1 && Q4.x == Q4.w && Q4.y == Q4.z) ? 0.5 : 1.0;
    for (int w = threadIdx.x; w < 2 * nla * 2 * nld; w += blockDim.x) {
      int a = w / (2 * nld), d = w % (2 * nld);
      double2 v = Kl[a * MAXSP + d];
      if (v.x == 0.0 && v.y == 0.0) continue;
      v.x *= wq; v.y *= wq;
      int fa = A.fock[a >> 1][a & 1] + oa, fdd = Dd.fock[d >> 1][d & 1] + od;
      double *dst = q.BX + 2 * ((size_t)fa + (size_t)q.ldf * fdd);
      atomicAdd(dst, v.x);
      atomicAdd(dst + 1, v.y);
    }
    if (dual)
      for (int w = threadIdx.x; w < 2 * nlc * 2 * nlb; w += blockDim.x) {
        int cc = w / (2 * nlb), b = w % (2 * nlb);
        double2 v = K2[cc * MAXSP + b];
        if (v.x == 0.0 && v.y == 0.0) continue;
        v.x *= wq; v.y *= wq;
        int fcc = C.fock[cc >> 1][cc & 1] + oc, fbb = B.fock[b >> 1][b & 1] + ob;
        double *dst = q.BX + 2 * ((size_t)fcc + (size_t)q.ldf * fbb);
        atomicAdd(dst, v.x);
        atomicAdd(dst + 1, v.y);
      }
    __syncthreads();
  }
}

// BXCH(J,I) = conj(BXCH(I,J)) for I in the large and J in the small block
// (BRTFAST :17643-17654).  One thread per element of the n x n LS block.
__global__ void k_conj_block(double2 *M, int n, int ld) {
  long long tot = (long long)n * n;
  for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < tot;
       w += (long long)gridDim.x * blockDim.x) {
    int i = int(w % n), j = int(w / n);
    double2 v = M[(size_t)i + (size_t)ld * (j + n)];
    M[(size_t)(j + n) + (size_t)ld * i] = make_double2(v.x, -v.y);
  }
}

// ---------------------------------------------------------------------------
// Split-precision (double-float) path.
// Every FP64 value v is carried as a pair of FP32 words (h, l), v = h + l,
// |l| <= ulp(h)/2, about 48 significant bits.  Products are formed exactly
// with FMA (TwoProd) and sums with TwoSum, so the contractions run on the
// FP32 pipes at ~2^-44 relative accuracy.  Boys values, the R recursion and
// the J/K accumulation stay FP64.  FP32's exponent range is kept by exact
// power-of-two scaling: E-coefficients of a pair with exponent sum p are
// stored times 2^(k_p*lambda), k_p = floor(log2(2p)/2); a quartet with
// reduced exponent alpha uses k = floor(log2(2 alpha)/2) <= k_p, k_q and
// rescales by 2^((k-k_p)lambda) (<= 1), R by 2^(-k lambda).
// ---------------------------------------------------------------------------
__host__ __device__ inline int half_floor_log2(double x) {
  int e = ilogb(x);
  return e >= 0 ? e / 2 : -((-e + 1) / 2);
}

__device__ inline void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// (sh, sl) += (ah + al) * (bh + bl)
__device__ inline void df_fma(float ah, float al, float bh, float bl, float &sh, float &sl) {
  float p = ah * bh;
  float pe = fmaf(ah, bh, -p);
  pe = fmaf(ah, bl, pe);
  pe = fmaf(al, bh, pe);
  float s, e;
  two_sum(sh, p, s, e);
  sh = s;
  sl += e + pe;
}

// (h, l) = (ah + al) + sgn * (bh + bl), renormalised
__device__ inline void df_add(float ah, float al, float bh, float bl, float &h, float &l) {
  float s, e;
  two_sum(ah, bh, s, e);
  e += al + bl;
  h = s + e;
  l = e - (h - s);
}

__device__ inline void df_split(double v, float &h, float &l) {
  h = __double2float_rn(v);
  l = __double2float_rn(v - (double)h);
}

__device__ inline double df_val(float h, float l) { return (double)h + (double)l; }

// Double-float copy of the E-coefficients, scaled per pair.
__global__ void k_econv(const double2 *E, float4 *Edf, const PairE *pe, const Shell *sh,
                        int ns, int ncomp) {
  long long pair = blockIdx.x;
  if (pair >= (long long)ns * ns) return;
  const Shell &A = sh[pair / ns], &B = sh[pair % ns];
  int k = pe[pair].kexp;
  int nl = (2 * A.l + 1) * (2 * B.l + 1);
  for (int comp = 0; comp < ncomp; ++comp) {
    int nt = ntuv(A.l + B.l + 2 * comp);
    long long off = pe[pair].off[comp];
    for (int w = threadIdx.x; w < nl * 2 * nt; w += blockDim.x) {
      int t = w % nt;
      int lam = c_t[t] + c_u[t] + c_v[t];
      double2 v = E[off + w];
      float4 o;
      df_split(ldexp(v.x, k * lam), o.x, o.y);
      df_split(ldexp(v.y, k * lam), o.z, o.w);
      Edf[off + w] = o;
    }
  }
}

// FP32 (re, im) copy of the double-float E copy (its high words): the
// tensor-core kernel's operand source, half the bytes.
__global__ void k_ef(const float4 *Edf, float2 *Ef, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    float4 v = Edf[i];
    Ef[i] = make_float2(v.x, v.z);
  }
}

// FP32 copy of the sigma-coupled LS/SL E-coefficients, one block per (pair,
// component), each coefficient times 2^(kexp lambda) (layout
// [lab_a][lab_b][set][x,y,z][tuv], degree l_a + l_b + 1).
__global__ void k_ebf(const double2 *EB, float2 *EBf, const long long *offq, const PairE *pe,
                      const Shell *sh, int ns) {
  long long pc = blockIdx.x;
  if (pc >= (long long)ns * ns * 2) return;
  long long pair = pc / 2;
  const Shell &A = sh[pair / ns], &B = sh[pair % ns];
  int k = pe[pair].kexp;
  int nt = ntuv(A.l + B.l + 1);
  long long n = (long long)(2 * A.l + 1) * (2 * B.l + 1) * 6 * nt, off = offq[pc];
  for (long long w = threadIdx.x; w < n; w += blockDim.x) {
    int t = (int)(w % nt);
    int lam = c_t[t] + c_u[t] + c_v[t];
    double2 v = EB[off + w];
    EBf[off + w] = make_float2(__double2float_rn(ldexp(v.x, k * lam)),
                               __double2float_rn(ldexp(v.y, k * lam)));
  }
}

// Double-float copy of the density (column-major, leading dimension ld).
__global__ void k_dconv(const double2 *D, int ld, int n, float4 *Ddf) {
  long long tot = (long long)n * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot;
       i += (long long)gridDim.x * blockDim.x) {
    long long r = i % n, c = i / n;
    double2 v = D[r + (long long)ld * c];
    float4 o;
    df_split(v.x, o.x, o.y);
    df_split(v.y, o.z, o.w);
    Ddf[r + (long long)n * c] = o;
  }
}

// Boys table for the split path: F_m(T_i) on T_i = i/32, 0 <= T_i <= 17,
// m < NBORD; F_m(T) from a 7-term Taylor expansion about the nearest point
// (|T-T_i| <= 1/64, truncation below 1e-16).  The FP64 path keeps the
// reference's 60-term series.
constexpr int NBGRID = 17 * 32 + 1;
constexpr int NBORD = MAXLAM + 7;
__device__ double g_boys_tab[NBGRID * NBORD];

__global__ void k_boys_table() {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NBGRID) return;
  double T = i / 32.0, F[NBORD];
  int top = NBORD - 1;
  double txp = exp(-T), tt2 = 2.0 * T, term = 1.0, s = 1.0;
  for (int k = 1; k <= 120; ++k) {
    term = term * tt2 / double(2 * top + 2 * k + 1);
    s += term;
  }
  F[top] = s * txp / double(2 * top + 1);
  for (int m = top - 1; m >= 0; --m) F[m] = (tt2 * F[m + 1] + txp) / double(2 * m + 1);
  for (int m = 0; m < NBORD; ++m) g_boys_tab[i * NBORD + m] = F[m];
}

// F_m(T) for T <= 17 from the table (7-term Taylor expansion about the
// nearest grid point).
__device__ __forceinline__ double boys_tab_m(double T, int m) {
  int i = __double2int_rn(T * 32.0);
  double d = i / 32.0 - T;  // -(T - T_i)
  const double *f = g_boys_tab + i * NBORD + m;
  double v = f[6] * (1.0 / 720.0);
  v = fma(v, d, f[5] * (1.0 / 120.0));
  v = fma(v, d, f[4] * (1.0 / 24.0));
  v = fma(v, d, f[3] * (1.0 / 6.0));
  v = fma(v, d, f[2] * 0.5);
  v = fma(v, d, f[1]);
  return fma(v, d, f[0]);
}

// F_0 .. F_lam for T > 17 by upward recursion: the reference's rational
// seed up to 30, asymptotic beyond (FUNFM's regimes).
__device__ __forceinline__ void boys_large(double T, int lam, double *F) {
  const double A0 = 4.994501191201870e-1, B0 = 4.551838436668326e-1;
  const double PI12 = 1.7724538509055160;
  if (T <= 30.0) {
    double txp = exp(-T), r2 = 0.5 / T;
    F[0] = 0.5 * PI12 / sqrt(T) - txp * (A0 / (B0 + T));
    for (int k = 0; k < lam; ++k) F[k + 1] = (double(2 * k + 1) * F[k] - txp) * r2;
  } else {
    double r2 = 0.5 / T;
    F[0] = 0.5 * PI12 / sqrt(T);
    for (int k = 0; k < lam; ++k) F[k + 1] = double(2 * k + 1) * F[k] * r2;
  }
}

// F_m(T) for m = threadIdx.x <= lam, all threads of the block take part
// (regimes as in FUNFM: exact at T=0, table below 17, the reference's
// rational seed up to 30, asymptotic beyond).
__device__ void boys_block(double T, int lam, double *F) {
  int m = threadIdx.x;
  if (T <= 1.0e-11) {
    if (m <= lam) F[m] = c_rinv[m];
  } else if (T <= 17.0) {
    if (m <= lam) F[m] = boys_tab_m(T, m);
  } else if (m == 0) {
    boys_large(T, lam, F);
  }
}

// Per-quartet scalars of a tensor-core launch, one thread per quartet for
// all quartets of the launch at once: the quartet geometry and Boys values
// are long dependent FP64 chains, which on one thread of each CTA would
// hold the whole CTA; here they run at full occupancy.  Record i of qp
// (QPW doubles):
//   [0..2] P - Q, [3] -2 alpha, [4] PRE = 2 pi^(5/2) / (p q sqrt(p + q)),
//   [5] T = alpha |P - Q|^2, [6] 1 / (2 alpha), [7] floor(log2(2 alpha) / 2)
//   (the exponent-balancing shift), [8 + n] (-2 alpha)^n F_n(T) for
//   n <= lam (RMAKE's R^(n)_000 before the PRE factor),
// with alpha = p q / (p + q) and lam = la + lb + lc + ld + lextra.  The
// arithmetic is that of the per-CTA code it replaces, value for value.
constexpr int QPW = 8 + MAXLAM + 1;
// Tensor-core launches take their lists in pieces of at most QP_CHUNK
// quartets, the size of the record scratch (200 MB).
constexpr long long QP_CHUNK = 1LL << 20;

// Hermite index of the sum of two Hermite terms, hidx(t_s + t_n, u_s + u_n,
// v_s + v_n), for n, s < NTE (row n holds NHS entries, the last ones
// unused): the gather table of the tensor-core kernels' Hankel operands.
constexpr int NHS = 192;
__device__ unsigned short g_hx[NTE * NHS];
__global__ void k_qprep(const Shell *sh, const int4 *quart, long long nq, int lextra,
                        double *qp) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nq;
       i += (long long)gridDim.x * blockDim.x) {
    int4 Q4 = quart[i];
    const Shell &A = sh[Q4.x], &B = sh[Q4.y], &C = sh[Q4.z], &Dd = sh[Q4.w];
    int lam = A.l + B.l + C.l + Dd.l + lextra;
    double p = A.alpha + B.alpha, qq = C.alpha + Dd.alpha;
    double Px = (A.alpha * A.x + B.alpha * B.x) / p;
    double Py = (A.alpha * A.y + B.alpha * B.y) / p;
    double Pz = (A.alpha * A.z + B.alpha * B.z) / p;
    double Qx = (C.alpha * C.x + Dd.alpha * Dd.x) / qq;
    double Qy = (C.alpha * C.y + Dd.alpha * Dd.y) / qq;
    double Qz = (C.alpha * C.z + Dd.alpha * Dd.z) / qq;
    double aph = p * qq / (p + qq);
    double T = aph * ((Qx - Px) * (Qx - Px) + (Qy - Py) * (Qy - Py) + (Qz - Pz) * (Qz - Pz));
    double *o = qp + i * QPW;
    o[0] = Px - Qx; o[1] = Py - Qy; o[2] = Pz - Qz;
    double m2a = -2.0 * aph;
    o[3] = m2a;
    o[4] = 2.0 * 17.493418327624863 / (sqrt(p + qq) * p * qq);
    o[5] = T;
    o[6] = 0.5 / aph;
    o[7] = (double)half_floor_log2(2.0 * aph);
    double F[MAXLAM + 1];
    if (T <= 1.0e-11) {
      for (int m = 0; m <= lam; ++m) F[m] = c_rinv[m];
    } else if (T <= 17.0) {
      for (int m = 0; m <= lam; ++m) F[m] = boys_tab_m(T, m);
    } else {
      boys_large(T, lam, F);
    }
    double pw = 1.0;
    for (int n = 0; n <= lam; ++n) {
      o[8 + n] = pw * F[n];
      pw *= m2a;
    }
  }
}

constexpr int CHDF = 2;  // most left labels per first-contraction pass (df path)
constexpr int DFTHREADS = 128;  // 4 quartets in flight per SM

// Left labels per pass: 2 for explicit lists; 1 when both quartet orders
// are digested (sym), whose contribution buffer holds twice the targets, so
// that both modes stay under 48 KB of shared memory and four CTAs per SM.
__host__ __device__ constexpr int df_chunk(int sym) { return sym ? 1 : CHDF; }

// contribution buffer (float4): chunk labels x MAXLAB^2 label pairs x targets
__host__ __device__ constexpr int df_ncb(int sym) {
  return df_chunk(sym) * MAXLAB * MAXLAB * (sym ? 16 : 8);
}

// doubles at the start of the df kernel's shared memory: R (FP64) or the
// contribution buffer, whichever is larger (even, so what follows stays
// 16-byte aligned)
__host__ __device__ constexpr int df_region0(int sym) {
  return df_ncb(sym) * 2 > NTR ? df_ncb(sym) * 2 : NTR + 1;
}

struct QArgsDF {
  const Shell *sh;
  const PairE *pe;
  const float4 *E;
  const unsigned char *Eci;  // Hermite indices of the nonzero E terms (k_ecompact)
  const float4 *D;  // n x n, leading dimension n (batched: the Inst placement)
  double *GD, *GX;
  int ns, ldd, ldf, nskp, isym, racah1;
  int sym;  // 1: also digest the swapped quartet (cd|ab) = (ab|cd) when ab != cd;
            // 2: as 1, lists halved by (ba|dc) = (ab|cd)* (weights, completion)
  const Inst *inst;  // batched build: per-instance placement (shell .inst), else null
};

// complex double-float product accumulate: (acc) += u * v
struct cdf { float rh, rl, ih, il; };

__device__ inline void cdf_mac(cdf &acc, float4 u, float4 v) {
  // re += u.re v.re - u.im v.im ; im += u.re v.im + u.im v.re
  df_fma(u.x, u.y, v.x, v.y, acc.rh, acc.rl);
  df_fma(-u.z, -u.w, v.z, v.w, acc.rh, acc.rl);
  df_fma(u.x, u.y, v.z, v.w, acc.ih, acc.il);
  df_fma(u.z, u.w, v.x, v.y, acc.ih, acc.il);
}

// (ab|cd) m-sign combination (sa,sb,sc,sd) of a label quartet from the
// eight contractions sv[0..7] = s1, s1c, s2, s2c, s3, s3c, s4, s4c of the
// (left|right) evaluation (ERIFAST :12809-13119): combination index
// 8a+4b+2c+d of (left|right); odd indices are conjugates; signs from the
// left pair phase sl and the product phase slr.
template <bool SWP>
__device__ inline float4 rv_sign(const float4 (&sv)[8], int sa, int sb, int sc, int sd,
                                 float sl, float slr) {
  int idx = SWP ? 8 * sc + 4 * sd + 2 * sa + sb : 8 * sa + 4 * sb + 2 * sc + sd;
  // source contraction and sign kind per index: kind 0 -> 1, 1 -> sl,
  // 2 -> slr, 3 -> sl*slr; negative kinds flip the sign
  const int src[16] = {0, 3, 2, 1, 5, 6, 7, 4, 4, 7, 6, 5, 1, 2, 3, 0};
  const int kind[16] = {0, -3, 0, 3, -1, 2, -1, -2, 0, -3, 0, 3, 1, -2, 1, 2};
  int kd = kind[idx];
  float f = 1.f;
  int ak = kd < 0 ? -kd : kd;
  if (ak == 1) f = sl;
  else if (ak == 2) f = slr;
  else if (ak == 3) f = sl * slr;
  if (kd < 0) f = -f;
  float4 v = sv[src[idx]];
  if (idx & 1) return make_float4(f * v.x, f * v.y, -f * v.z, -f * v.w);
  return make_float4(f * v.x, f * v.y, f * v.z, f * v.w);
}

__global__ void __launch_bounds__(DFTHREADS, 4)
k_quartet_df(QArgsDF q, const int4 *quart, long long nq, int t1, int t2) {
  // Shared memory (sizes in df_smem_layout): the FP64 R-integrals are dead
  // once their double-float copy Rf exists, so the contribution buffer Cb
  // (J, K and, with sym, J2, K2: 4 targets each per label quartet) shares
  // their space; R2, the recursion's second buffer, shares Rf's.
  extern __shared__ double smem[];
  const int r0d = df_region0(q.sym);
  const int ch = df_chunk(q.sym);              // left labels per pass
  double *R = smem;                            // NTR (FP64)
  float4 *Cb = (float4 *)smem;                 // df_ncb(sym)
  float2 *Rf = (float2 *)(smem + r0d);         // NTR (df), padded to NTR+1 doubles
  double *R2 = (double *)Rf;                   // FP64 recursion buffer (aliases Rf)
  double *F = smem + r0d + NTR + 1;            // MAXLAM+2
  float4 *EL = (float4 *)(F + MAXLAM + 2);     // ch*2*NTE
  float4 *G = EL + ch * 2 * NTE;               // ch*2*NTE
  double2 *Jl = (double2 *)(G + ch * 2 * NTE);  // MAXSP*MAXSP
  double2 *Kl = Jl + MAXSP * MAXSP;
  double2 *J2 = Kl + MAXSP * MAXSP;            // with sym only
  double2 *K2 = J2 + MAXSP * MAXSP;
  __shared__ unsigned char ELi[CHDF * 2 * NTE];  // Hermite indices of the staged E
  __shared__ double sgeo[8];
  __shared__ int sk;

  for (long long qi = blockIdx.x; qi < nq; qi += gridDim.x) {
    int4 Q4 = quart[qi];
    const Shell &A = q.sh[Q4.x], &B = q.sh[Q4.y], &C = q.sh[Q4.z], &Dd = q.sh[Q4.w];
    int la = A.l, lb = B.l, lc = C.l, ld = Dd.l;
    int degab = la + lb + 2 * t1, degcd = lc + ld + 2 * t2;
    int lam = degab + degcd;
    int nla = 2 * la + 1, nlb = 2 * lb + 1, nlc = 2 * lc + 1, nld = 2 * ld + 1;
    int nlab = nla * nlb, nlcd = nlc * nld;
    int nab = ntuv(degab), ncd = ntuv(degcd);
    bool swp = contraction_cost(nlcd, ncd, nlab, nab) < contraction_cost(nlab, nab, nlcd, ncd);
    int mcnt = ncntrs(A.cnt, B.cnt, C.cnt, Dd.cnt);
    // matrix placement: the call's arrays, or this quartet's instance in a batch
    const float4 *Dm = q.D;
    double *GDm = q.GD, *GXm = q.GX;
    size_t lddm = q.ldd, ldfm = q.ldf;
    int nskpm = q.nskp;
    if (q.inst) {
      const Inst I = q.inst[A.inst];
      if (Dm) Dm += I.off;
      if (GDm) { GDm += 2 * I.off; GXm += 2 * I.off; }
      lddm = ldfm = (size_t)I.ld;
      nskpm = I.nskp;
    }
    const PairE &pab_e = q.pe[A.prow + Q4.y], &pcd_e = q.pe[C.prow + Q4.w];
    if (threadIdx.x == 0) {
      double p = A.alpha + B.alpha, qq = C.alpha + Dd.alpha;
      double Px = (A.alpha * A.x + B.alpha * B.x) / p;
      double Py = (A.alpha * A.y + B.alpha * B.y) / p;
      double Pz = (A.alpha * A.z + B.alpha * B.z) / p;
      double Qx = (C.alpha * C.x + Dd.alpha * Dd.x) / qq;
      double Qy = (C.alpha * C.y + Dd.alpha * Dd.y) / qq;
      double Qz = (C.alpha * C.z + Dd.alpha * Dd.z) / qq;
      double aph = p * qq / (p + qq);
      double T = aph * ((Qx - Px) * (Qx - Px) + (Qy - Py) * (Qy - Py) + (Qz - Pz) * (Qz - Pz));
      double sg = swp ? -1.0 : 1.0;
      sgeo[0] = sg * (Px - Qx); sgeo[1] = sg * (Py - Qy); sgeo[2] = sg * (Pz - Qz);
      sgeo[3] = -2.0 * aph;
      sgeo[4] = 2.0 * 17.493418327624863 / (sqrt(p + qq) * p * qq);
      sgeo[5] = T;
      sk = half_floor_log2(2.0 * aph);
    }
    __syncthreads();
    boys_block(sgeo[5], lam, F);
    __syncthreads();
    {
      double X = sgeo[0], Y = sgeo[1], Z = sgeo[2], m2a = sgeo[3];
      double *cur = R, *nxt = R2;
      for (int n = lam; n >= 0; --n) {
        int cnt = ntuv(lam - n);
        for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
          double val;
          if (k == 0) {
            double pw = 1.0;
            for (int i = 0; i < n; ++i) pw *= m2a;
            val = pw * F[n];
          } else {
            int t = c_t[k], u = c_u[k], v = c_v[k];
            if (t > 0) {
              val = X * cur[hidx(t - 1, u, v)];
              if (t > 1) val += double(t - 1) * cur[hidx(t - 2, u, v)];
            } else if (u > 0) {
              val = Y * cur[hidx(t, u - 1, v)];
              if (u > 1) val += double(u - 1) * cur[hidx(t, u - 2, v)];
            } else {
              val = Z * cur[hidx(t, u, v - 1)];
              if (v > 1) val += double(v - 1) * cur[hidx(t, u, v - 2)];
            }
          }
          nxt[k] = val;
        }
        __syncthreads();
        double *tmp = cur; cur = nxt; nxt = tmp;
      }
      // scaled double-float copy of PRE*R (R2 and Rf alias: go through R)
      double pre = sgeo[4];
      int nt = ntuv(lam);
      if (cur != R) {
        for (int k = threadIdx.x; k < nt; k += blockDim.x) R[k] = cur[k];
        __syncthreads();
      }
      int k = sk;
      for (int i = threadIdx.x; i < nt; i += blockDim.x) {
        int L = c_t[i] + c_u[i] + c_v[i];
        float h, l;
        df_split(ldexp(R[i] * pre, -k * L), h, l);
        Rf[i] = make_float2(h, l);
      }
    }
    for (int i = threadIdx.x; i < MAXSP * MAXSP; i += blockDim.x) {
      Jl[i] = make_double2(0.0, 0.0);
      Kl[i] = make_double2(0.0, 0.0);
      if (q.sym) {
        J2[i] = make_double2(0.0, 0.0);
        K2[i] = make_double2(0.0, 0.0);
      }
    }
    __syncthreads();  // R is dead from here on: Cb may overwrite it
    bool dual = q.sym && (Q4.x != Q4.z || Q4.y != Q4.w || t1 != t2);
    int ntg = dual ? 16 : 8;
    const float4 *Eab = q.E + pab_e.off[t1];
    const float4 *Ecd = q.E + pcd_e.off[t2];
    const float4 *EGL = swp ? Ecd : Eab, *ER = swp ? Eab : Ecd;
    const unsigned char *EGi = q.Eci + (swp ? pcd_e.off[t2] : pab_e.off[t1]);
    const unsigned char *ERi = q.Eci + (swp ? pab_e.off[t1] : pcd_e.off[t2]);
    int kL = swp ? pcd_e.kexp : pab_e.kexp, kR = swp ? pab_e.kexp : pcd_e.kexp;
    int nL = swp ? ncd : nab, nR = swp ? nab : ncd;
    int nlL = swp ? nlcd : nlab, nlR = swp ? nlab : nlcd;
    int nl2L = swp ? nld : nlb, nl2R = swp ? nlb : nld;
    int lq[4] = {la, lb, lc, ld};
    int oab = t1 ? nskpm : 0, ocd = t2 ? nskpm : 0;
    int kq0 = sk;
    __syncthreads();
    // left labels per pass: as many as the staging buffers (EL and G,
    // ch*2*NTE float4 each) and the contribution buffer (df_ncb) take at
    // this class's degrees; ch at the largest degree, more for low l
    int chunk = min((ch * 2 * NTE) / (2 * max(nL, nR)), df_ncb(q.sym) / (nlR * ntg));
    chunk = max(1, chunk);
    for (int c0 = 0; c0 < nlL; c0 += chunk) {
      int nch = min(chunk, nlL - c0);
      // stage the nonzero left E-coefficients (packed, with their Hermite
      // indices) rescaled to this quartet's exponent
      for (int w = threadIdx.x; w < nch * 2 * nL; w += blockDim.x) {
        long long g = (long long)c0 * 2 * nL + w;
        int s = EGi[g];
        ELi[w] = (unsigned char)s;
        if (s == ENDIDX) continue;
        int L = c_t[s] + c_u[s] + c_v[s];
        float4 v = EGL[g - (w % nL) + s];
        float f = ldexpf(1.0f, (kq0 - kL) * L);
        EL[w] = make_float4(v.x * f, v.y * f, v.z * f, v.w * f);
      }
      __syncthreads();
      // first contraction G[lab][set][q] = Z(q) 2^((k-kR)lq) sum_s E_L R'[s+q]
      for (int w = threadIdx.x; w < nch * 2 * nR; w += blockDim.x) {
        int ls = w / nR, qq = w % nR;
        const float4 *e = EL + ls * nL;
        const unsigned char *ei = ELi + ls * nL;
        int tq = c_t[qq], uq = c_u[qq], vq = c_v[qq];
        float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
        for (int k = 0; k < nL; ++k) {
          int s = ei[k];
          if (s == ENDIDX) break;
          float2 rv = Rf[hidx(c_t[s] + tq, c_u[s] + uq, c_v[s] + vq)];
          float4 ev = e[k];
          df_fma(ev.x, ev.y, rv.x, rv.y, rh, rl);
          df_fma(ev.z, ev.w, rv.x, rv.y, ih, il);
        }
        int lq_ = tq + uq + vq;
        float f = ldexpf((lq_ & 1) ? -1.0f : 1.0f, (kq0 - kR) * lq_);
        G[ls * nR + qq] = make_float4(rh * f, rl * f, ih * f, il * f);
      }
      __syncthreads();
      {
        // each label quartet's second contraction is split over KS lanes
        // (more lanes for classes with few label quartets) and summed with a
        // butterfly of shuffles; the KS lanes then share its 8 J/K targets
        int items = nch * nlR;
        int KS = 1;
        while (KS < 8 && items * KS * 2 <= (int)blockDim.x) KS *= 2;
        int lanes = items * KS;
        for (int base = 0; base < lanes; base += blockDim.x) {
          int t = base + threadIdx.x;
          bool valid = t < lanes;
          int item = valid ? t / KS : 0, part = t % KS;
          int lab = item / nlR, lr = item % nlR;
          int labL = c0 + lab;
          int l1 = labL / nl2L, l2 = labL % nl2L, r1 = lr / nl2R, r2 = lr % nl2R;
          int ia = swp ? r1 : l1, ib = swp ? r2 : l2, ic = swp ? l1 : r1, id = swp ? l2 : r2;
          int kq[4], mq[4], mm[4];
          label_of(la, ia, kq[0], mm[0]);
          label_of(lb, ib, kq[1], mm[1]);
          label_of(lc, ic, kq[2], mm[2]);
          label_of(ld, id, kq[3], mm[3]);
          for (int i = 0; i < 4; ++i) mq[i] = 2 * mm[i] - 1;
          bool active = valid && label_ok(q.isym, q.racah1, mcnt, kq, mq, lq);
          float acc[16][2];
#pragma unroll
          for (int i = 0; i < 16; ++i) { acc[i][0] = 0.f; acc[i][1] = 0.f; }
          if (active) {
            const float4 *g11 = G + (lab * 2 + 0) * nR, *g21 = G + (lab * 2 + 1) * nR;
            const float4 *e11 = ER + ((long long)lr * 2 + 0) * nR;
            const float4 *e21 = ER + ((long long)lr * 2 + 1) * nR;
            // right-side E from L2 with one iteration of register prefetch
            float4 u1n = make_float4(0.f, 0.f, 0.f, 0.f), u2n = u1n;
            if (part < nR) { u1n = e11[part]; u2n = e21[part]; }
            if (q.isym) {
              // CLMMTZ reads only the real parts of combinations 0, 3, 12,
              // 15 and 0, 6, 9, 15: products (e11 x g11) and (e21 x g21),
              // real-by-real and imaginary-by-imaginary (ERIFAST :12820-12912),
              // over the nonzero E terms of each set
              const unsigned char *i1 = ERi + (long long)lr * 2 * nR, *i2 = i1 + nR;
              for (int k = part; k < nR; k += KS) {
                int kk = i1[k];
                if (kk == ENDIDX) break;
                float4 u1 = e11[kk], x1 = g11[kk];
                df_fma(u1.x, u1.y, x1.x, x1.y, acc[0][0], acc[0][1]);
                df_fma(u1.z, u1.w, x1.z, x1.w, acc[1][0], acc[1][1]);
              }
              for (int k = part; k < nR; k += KS) {
                int kk = i2[k];
                if (kk == ENDIDX) break;
                float4 u2 = e21[kk], x2 = g21[kk];
                df_fma(u2.x, u2.y, x2.x, x2.y, acc[12][0], acc[12][1]);
                df_fma(u2.z, u2.w, x2.z, x2.w, acc[13][0], acc[13][1]);
              }
            } else
            for (int k = part; k < nR; k += KS) {
              float4 u1 = u1n, u2 = u2n;
              if (k + KS < nR) { u1n = e11[k + KS]; u2n = e21[k + KS]; }
              float4 x1 = g11[k], x2 = g21[k];
#define P4(o, UU, XX)                                           \
  df_fma(UU.x, UU.y, XX.x, XX.y, acc[o][0], acc[o][1]);         \
  df_fma(UU.z, UU.w, XX.z, XX.w, acc[o + 1][0], acc[o + 1][1]); \
  df_fma(UU.x, UU.y, XX.z, XX.w, acc[o + 2][0], acc[o + 2][1]); \
  df_fma(UU.z, UU.w, XX.x, XX.y, acc[o + 3][0], acc[o + 3][1]);
              P4(0, u1, x1) P4(4, u2, x1) P4(8, u1, x2) P4(12, u2, x2)
#undef P4
            }
          }
          for (int off = KS >> 1; off > 0; off >>= 1) {
#pragma unroll
            for (int i = 0; i < 16; ++i) {
              float oh = __shfl_xor_sync(0xffffffffu, acc[i][0], off);
              float ol = __shfl_xor_sync(0xffffffffu, acc[i][1], off);
              df_add(acc[i][0], acc[i][1], oh, ol, acc[i][0], acc[i][1]);
            }
          }
          if (!valid) continue;
          float4 *cb = Cb + (size_t)(lab * nlR + lr) * ntg;
          if (!active) {
            for (int tg = part; tg < ntg; tg += KS) cb[tg] = make_float4(0.f, 0.f, 0.f, 0.f);
            continue;
          }
          double pab = pair_phase(kq[0], mm[0], kq[1], mm[1]);
          double pcd = pair_phase(kq[2], mm[2], kq[3], mm[3]);
          double pl = swp ? pcd : pab, pr = swp ? pab : pcd;
          // s = u*x = (a-b, c+d) ; sc = u*conj(x) = (a+b, d-c)
          float4 sv[8];
#pragma unroll
          for (int pp = 0; pp < 4; ++pp) {
            float *a = acc[4 * pp], *b = acc[4 * pp + 1], *c = acc[4 * pp + 2], *d = acc[4 * pp + 3];
            float4 tt, tc;
            df_add(a[0], a[1], -b[0], -b[1], tt.x, tt.y);
            df_add(c[0], c[1], d[0], d[1], tt.z, tt.w);
            df_add(a[0], a[1], b[0], b[1], tc.x, tc.y);
            df_add(d[0], d[1], -c[0], -c[1], tc.z, tc.w);
            sv[2 * pp] = tt;
            sv[2 * pp + 1] = tc;
          }
          float sl_ = pl < 0 ? -1.f : 1.f, slr = (pl * pr) < 0 ? -1.f : 1.f;
          int fa[2] = {A.fock[ia][0] + oab, A.fock[ia][1] + oab};
          int fb[2] = {B.fock[ib][0] + oab, B.fock[ib][1] + oab};
          int fc[2] = {C.fock[ic][0] + ocd, C.fock[ic][1] + ocd};
          int fd[2] = {Dd.fock[id][0] + ocd, Dd.fock[id][1] + ocd};
          const size_t ld = lddm;
          // phase A: targets tg = 4*family + sig.  family 0 J(a,b) sig=(sa,sb),
          // 1 K(a,d) sig=(sa,sd), 2 J(c,d) of (cd|ab) sig=(sc,sd),
          // 3 K(c,b) of (cd|ab) sig=(sc,sb)
#pragma unroll 1
          for (int tg = part; tg < ntg; tg += KS) {
            int fam = tg >> 2, s1 = (tg >> 1) & 1, s2 = tg & 1;
            cdf o = {0.f, 0.f, 0.f, 0.f};
            if (q.isym == 0) {
#pragma unroll
              for (int x = 0; x < 2; ++x)
#pragma unroll
                for (int y = 0; y < 2; ++y) {
                  int sa, sb, sc2, sd;
                  float4 dv;
                  if (fam == 0) {
                    sa = s1; sb = s2; sc2 = x; sd = y; dv = Dm[fc[sc2] + ld * fd[sd]];
                  } else if (fam == 1) {
                    sa = s1; sd = s2; sb = x; sc2 = y; dv = Dm[fc[sc2] + ld * fb[sb]];
                  } else if (fam == 2) {
                    sc2 = s1; sd = s2; sa = x; sb = y; dv = Dm[fa[sa] + ld * fb[sb]];
                  } else {
                    sc2 = s1; sb = s2; sa = x; sd = y; dv = Dm[fa[sa] + ld * fd[sd]];
                  }
                  float4 v = swp ? rv_sign<true>(sv, sa, sb, sc2, sd, sl_, slr)
                                 : rv_sign<false>(sv, sa, sb, sc2, sd, sl_, slr);
                  cdf_mac(o, v, dv);
                }
            } else if (s1 == s2) {
              // CLMMTZ: real parts, equal-sign direct blocks, crossed exchange
              int sg = s1;
#pragma unroll
              for (int tt = 0; tt < 2; ++tt) {
                int sa, sb, sc2, sd;
                float4 dv;
                if (fam == 0) {
                  sa = sg; sb = sg; sc2 = tt; sd = tt; dv = Dm[fc[tt] + ld * fd[tt]];
                } else if (fam == 1) {
                  sa = sg; sb = tt; sc2 = tt; sd = sg; dv = Dm[fc[tt] + ld * fb[tt]];
                } else if (fam == 2) {
                  sa = tt; sb = tt; sc2 = sg; sd = sg; dv = Dm[fa[tt] + ld * fb[tt]];
                } else {
                  sa = tt; sb = sg; sc2 = sg; sd = tt; dv = Dm[fa[tt] + ld * fd[tt]];
                }
                float4 v = swp ? rv_sign<true>(sv, sa, sb, sc2, sd, sl_, slr)
                               : rv_sign<false>(sv, sa, sb, sc2, sd, sl_, slr);
                df_fma(v.x, v.y, dv.x, dv.y, o.rh, o.rl);
              }
            }
            cb[tg] = make_float4(o.rh, o.rl, o.ih, o.il);
          }
        }
      }
      __syncthreads();
      // phase B: one thread per J or K target sums the chunk's contributions
      // in double-float and adds the FP64 value to the shared accumulator.
      // Families: 0 J(ia,ib), 1 K(ia,id), 2 J(ic,id), 3 K(ic,ib).  Only
      // targets that this chunk's left labels can reach are enumerated: an
      // index of the left pair ranges over the chunk's values, the others
      // over all labels.
      {
        int nfam = dual ? 4 : 2;
        int l1lo = c0 / nl2L, l1hi = (c0 + nch - 1) / nl2L;
        int l2lo = 0, l2hi = nl2L - 1;
        if (l1lo == l1hi) { l2lo = c0 % nl2L; l2hi = (c0 + nch - 1) % nl2L; }
        // label ranges of the roles a, b, c, d
        int rlo[4] = {0, 0, 0, 0}, rhi[4] = {nla - 1, nlb - 1, nlc - 1, nld - 1};
        int r1 = swp ? 2 : 0;
        rlo[r1] = l1lo; rhi[r1] = l1hi;
        rlo[r1 + 1] = l2lo; rhi[r1 + 1] = l2hi;
        const int fx[4] = {0, 0, 2, 2}, fy[4] = {1, 3, 3, 1};
        int tot = 0, start[5], ny[4];
        for (int f = 0; f < 4; ++f) {
          start[f] = tot;
          ny[f] = rhi[fy[f]] - rlo[fy[f]] + 1;
          if (f < nfam) tot += (rhi[fx[f]] - rlo[fx[f]] + 1) * ny[f] * 4;
        }
        start[4] = tot;
        for (int w = threadIdx.x; w < tot; w += blockDim.x) {
          int f = 0;
          while (w >= start[f + 1]) ++f;
          int u = w - start[f], sig = u & 3, tgt = u >> 2;
          int X = rlo[fx[f]] + tgt / ny[f], Y = rlo[fy[f]] + tgt % ny[f];
          float sh_r = 0.f, sl_r = 0.f, sh_i = 0.f, sl_i = 0.f;
          int cnt = 0;
          int fix[4] = {-1, -1, -1, -1};
          fix[fx[f]] = X;
          fix[fy[f]] = Y;
          // the left label is (l1,l2) = (ia,ib) or, swapped, (ic,id); the
          // right label likewise
          int fl1 = fix[r1], fl2 = fix[r1 + 1];
          int fr1 = fix[2 - r1], fr2 = fix[3 - r1];
          int q1lo = 0, q1hi = nlR / nl2R, q2lo = 0, q2hi = nl2R;
          if (fr1 >= 0) { q1lo = fr1; q1hi = fr1 + 1; }
          if (fr2 >= 0) { q2lo = fr2; q2hi = fr2 + 1; }
          for (int lab = 0; lab < nch; ++lab) {
            int labL = c0 + lab;
            int l1 = labL / nl2L, l2 = labL % nl2L;
            if ((fl1 >= 0 && l1 != fl1) || (fl2 >= 0 && l2 != fl2)) continue;
            for (int q1 = q1lo; q1 < q1hi; ++q1)
              for (int q2 = q2lo; q2 < q2hi; ++q2) {
                float4 v = Cb[(size_t)(lab * nlR + q1 * nl2R + q2) * ntg + 4 * f + sig];
                df_add(sh_r, sl_r, v.x, v.y, sh_r, sl_r);
                df_add(sh_i, sl_i, v.z, v.w, sh_i, sl_i);
                ++cnt;
              }
          }
          if (cnt) {
            double2 *acc2 = f == 0 ? Jl : (f == 1 ? Kl : (f == 2 ? J2 : K2));
            double2 *dst = &acc2[(X * 2 + (sig >> 1)) * MAXSP + Y * 2 + (sig & 1)];
            dst->x += df_val(sh_r, sl_r);
            dst->y += df_val(sh_i, sl_i);
          }
        }
      }
      __syncthreads();
    }
    // weight 1/2 for a quartet equal to its (ba|dc) image, or to its
    // (dc|ba) image within one class: the completion adds it again
    const double wq = (q.sym == 2 && ((Q4.x == Q4.y && Q4.z == Q4.w) ||
                                      (t1 == t2 && Q4.x == Q4.w && Q4.y == Q4.z))) ? 0.5 : 1.0;
    // flush shared accumulators (FP64)
    {
      int nsa = 2 * nla;
      for (int w = threadIdx.x; w < nsa * 2 * nlb; w += blockDim.x) {
        int a = w / (2 * nlb), b = w % (2 * nlb);
        double2 v = Jl[a * MAXSP + b];
        if (v.x == 0.0 && v.y == 0.0) continue;
        v.x *= wq; v.y *= wq;
        int fa = A.fock[a >> 1][a & 1] + oab, fbb = B.fock[b >> 1][b & 1] + oab;
        double *dst = GDm + 2 * ((size_t)fa + ldfm * fbb);
        atomicAdd(dst, v.x);
        atomicAdd(dst + 1, v.y);
      }
      for (int w = threadIdx.x; w < nsa * 2 * nld; w += blockDim.x) {
        int a = w / (2 * nld), d = w % (2 * nld);
        double2 v = Kl[a * MAXSP + d];
        if (v.x == 0.0 && v.y == 0.0) continue;
        v.x *= wq; v.y *= wq;
        int fa = A.fock[a >> 1][a & 1] + oab, fdd = Dd.fock[d >> 1][d & 1] + ocd;
        double *dst = GXm + 2 * ((size_t)fa + ldfm * fdd);
        atomicAdd(dst, v.x);
        atomicAdd(dst + 1, v.y);
      }
      if (dual) {
        int nsc = 2 * nlc;
        for (int w = threadIdx.x; w < nsc * 2 * nld; w += blockDim.x) {
          int c = w / (2 * nld), d = w % (2 * nld);
          double2 v = J2[c * MAXSP + d];
          if (v.x == 0.0 && v.y == 0.0) continue;
          v.x *= wq; v.y *= wq;
          int fcc = C.fock[c >> 1][c & 1] + ocd, fdd = Dd.fock[d >> 1][d & 1] + ocd;
          double *dst = GDm + 2 * ((size_t)fcc + ldfm * fdd);
          atomicAdd(dst, v.x);
          atomicAdd(dst + 1, v.y);
        }
        for (int w = threadIdx.x; w < nsc * 2 * nlb; w += blockDim.x) {
          int c = w / (2 * nlb), b = w % (2 * nlb);
          double2 v = K2[c * MAXSP + b];
          if (v.x == 0.0 && v.y == 0.0) continue;
          v.x *= wq; v.y *= wq;
          int fcc = C.fock[c >> 1][c & 1] + ocd, fbb = B.fock[b >> 1][b & 1] + oab;
          double *dst = GXm + 2 * ((size_t)fcc + ldfm * fbb);
          atomicAdd(dst, v.x);
          atomicAdd(dst + 1, v.y);
        }
      }
    }
    __syncthreads();
  }
}

// Hermitian completion G <- G + G^H of the n x n block(s) (CLMFAST's
// completion of a symmetry-reduced build, bertha-scf.f:12164-12205): one
// thread per element pair (i, j), i <= j.  With `inst`, block k of a batch
// (placement inst[k], size ndim[k]); else the one block at G, leading
// dimension ld.
__global__ void k_herm_complete(double2 *G, int n, long long ld, const Inst *inst,
                                const int *ndim, int ninst) {
  for (int k = blockIdx.x; k < ninst; k += gridDim.x) {
    double2 *M = G;
    long long m = n, l = ld;
    if (inst) {
      M = G + inst[k].off;
      m = ndim[k];
      l = inst[k].ld;
    }
    for (long long w = threadIdx.x + (long long)blockDim.x * blockIdx.y; w < m * m;
         w += (long long)blockDim.x * gridDim.y) {
      long long i = w % m, j = w / m;
      if (i > j) continue;
      double2 a = M[i + l * j];
      if (i == j) {
        M[i + l * j] = make_double2(2.0 * a.x, 0.0);
      } else {
        double2 b = M[j + l * i];
        double2 x = make_double2(a.x + b.x, a.y - b.y);
        M[i + l * j] = x;
        M[j + l * i] = make_double2(x.x, -x.y);
      }
    }
  }
}

// Zeroes the ndim x ndim block of every instance of a batched build.
__global__ void k_zero_inst(double *a, const Inst *inst, const int *ndim, int ninst) {
  for (int k = blockIdx.x; k < ninst; k += gridDim.x) {
    Inst I = inst[k];
    long long tot = (long long)ndim[k] * ndim[k];
    for (long long i = threadIdx.x + (long long)blockDim.x * blockIdx.y; i < tot;
         i += (long long)blockDim.x * gridDim.y) {
      long long r = i % ndim[k], c = i / ndim[k];
      double *p = a + 2 * (I.off + r + (long long)I.ld * c);
      p[0] = 0.0;
      p[1] = 0.0;
    }
  }
}

// Double-float copy of n consecutive complex elements (a batched density in
// the caller's placement).
__global__ void k_dconv1(const double2 *D, long long n, float4 *Ddf) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double2 v = D[i];
    float4 o;
    df_split(v.x, o.x, o.y);
    df_split(v.y, o.z, o.w);
    Ddf[i] = o;
  }
}

__global__ void k_zero2d(double *a, int n, int ld) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  long long tot = (long long)n * n;
  for (; i < tot; i += (long long)gridDim.x * blockDim.x) {
    long long r = i % n, c = i / n;
    a[2 * (r + (long long)ld * c)] = 0.0;
    a[2 * (r + (long long)ld * c) + 1] = 0.0;
  }
}

size_t quartet_smem_df(int sym) {
  return sizeof(double) * (df_region0(sym) + NTR + 1 + MAXLAM + 2) +
         sizeof(float4) * (2 * df_chunk(sym) * 2 * NTE) +
         sizeof(double2) * ((sym ? 4 : 2) * MAXSP * MAXSP);
}

// dynamic shared memory attribute of k_quartet_df: the larger mode
size_t quartet_smem_df_max() { return std::max(quartet_smem_df(0), quartet_smem_df(1)); }

size_t quartet_smem() {
  return sizeof(double) * (2 * NTR + MAXLAM + 2) + sizeof(double2) * (CHUNK * 2 * NTE + 4 * MAXSP * MAXSP);
}

}  // namespace

namespace {
#include "tc_quartet.cuh"

// Launch geometry of the tensor-core kernels for classes needing at most
// (n1, n2) TMEM columns for D1 and D2: the allocation (a power of two,
// 32..512; the Breit kernel keeps three D1 side by side when they fit, tri),
// the CTAs that share an SM's 512 columns (256 threads each, or one CTA of
// 512 threads), double buffering for a lone CTA when its shared memory
// fits, and a dynamic shared-memory request large enough that no more CTAs
// than that are resident on one SM (a surplus CTA would block in
// tcgen05.alloc until a neighbour exits).
struct TcGeom {
  int cols, ctas_per_sm, nbuf, nt, tri;
  size_t smem;
};
constexpr size_t SM_SMEM = 233472;  // 228 KB of shared memory per SM
constexpr size_t TC_SMEM_MAX = 232448;  // 227 KB, the per-CTA opt-in limit
size_t g_tc_smem_max = 122880;  // dynamic shared memory the tensor-core kernels may ask for

// f64acc: the Coulomb kernel's shared J/K accumulators in FP64 (Fock
// builds) or FP32 (explicit lists); the Breit kernel's are FP64.
TcGeom tc_geom(int n1, int n2, bool breit = false, bool f64acc = true) {
  TcGeom g;
  g.tri = breit && 3 * n1 + n2 <= 512 ? 1 : 0;
  int need = (g.tri ? 3 * n1 : n1) + n2, cols = 32;
  while (cols < need) cols *= 2;
  g.cols = cols;
  auto total = [&](int nb) {
    return breit ? (size_t)tcq::layout_b(n1, n2, nb, g.tri).total
                 : (size_t)tcq::layout_c(n1, n2, nb, f64acc).total;
  };
  size_t s = total(1);
  int ctas = std::min(2, 512 / cols);
  while (ctas > 1 && (s + 1024 + 4096) * ctas > SM_SMEM) --ctas;  // + static shared memory
  g.nbuf = 1;
  if (ctas == 1 && total(2) <= g_tc_smem_max) {
    g.nbuf = 2;
    s = total(2);
  }
  g.nt = ctas == 1 ? 512 : 256;
  // smallest request that still keeps ctas + 1 CTAs off one SM
  size_t floor_req = SM_SMEM / (ctas + 1) - 1024 + 64;
  g.smem = std::max(s, floor_req);
  g.ctas_per_sm = ctas;
  return g;
}
}  // namespace

// ---------------------------------------------------------------------------
// Context and C ABI
// ---------------------------------------------------------------------------
// A run of consecutive entries of a quartet list and the kernel that
// digests it under BG_PREC_AUTO (df: the split-precision kernel).
enum { KIND_FP64 = 0, KIND_DF32 = 1, KIND_TC = 2 };

// One row of the tuner's record: segment, class, sample time per kernel,
// estimated error per kernel, choice.
struct TuneRow {
  int comp, key;
  long long start, n;
  float t[3];
  double err[3];
  int kind;
};
struct Run {
  long long start, count;
  int kind;    // KIND_*: the kernel that digests this run
  int n1, n2;  // KIND_TC: largest TMEM column needs (D1, D2) of the run's classes
};

struct bg_ctx {
  int dev = -1;  // device the context was made on
  int ncnt = 0, ndim = 0, nskp = 0, hmlt = 0, isym = 0, racah1 = 1;
  std::vector<double> cxyz;  // BXYZ of the centres
  int ns = 0, ncomp = 1;
  std::vector<Shell> shells;
  std::vector<int> lmax;
  std::vector<int> lrge;  // [cnt][2*MAXLB+2][28]
  Shell *d_sh = nullptr;
  PairE *d_pe = nullptr;
  double2 *d_E = nullptr;
  long long nE = 0;
  double2 *d_Ecv = nullptr;        // sparse copies of d_E (k_ecompact)
  unsigned char *d_Eci = nullptr;
  // quartet lists for the Fock build, one per (t1,t2) component class
  int *d_quart[4] = {nullptr, nullptr, nullptr, nullptr};
  long long nquart[4] = {0, 0, 0, 0};
  int quart_ilev = -1;
  // lists too large to keep: regenerated every build and streamed in chunks
  // through two pinned host and two device buffers
  bool stream_lists = false;
  long long cache_q = 0, chunk_q = 0;  // limits in quartets (0: defaults)
  int *h_chunk[2] = {nullptr, nullptr}, *d_chunk[2] = {nullptr, nullptr};
  cudaEvent_t chunk_ev[2] = {nullptr, nullptr};
  double screen = 0.0;          // Schwarz threshold on Q_ab*Q_cd, 0 = off
  std::vector<double> qbound;   // [pair*2+comp] sqrt max |(ab|ab)|
  double2 *d_D = nullptr, *d_GD = nullptr, *d_GX = nullptr;
  // BG_PREC_AUTO: angular-class segments of the cached lists and the tuned
  // kernel of each run of them (see tune_runs)
  std::vector<long long> seg[4];
  std::vector<int> segkey[4];  // angular class (la,lb,lc,ld) of each segment, base 4
  std::vector<Run> runs[4];
  bool tuned = false;
  // split-precision copies: double-float E (and density), FP32 E (re, im) for
  // the tensor-core kernel, both scaled by 2^(kexp lambda)
  float4 *d_Edf = nullptr, *d_Ddf = nullptr;
  double *d_qp = nullptr;  // k_qprep records of tensor-core launches (QP_CHUNK of them)
  float2 *d_Ef = nullptr;
  int prec = BG_PREC_FP64;
  double err_budget = 1e-7;  // BG_PREC_AUTO: estimated energy error allowed per build (Eh)
  // Breit: sigma-coupled LS/SL E-coefficients (generated on first use) and
  // quartet lists of the classes (LS|LS) and (LS|SL)
  int gaunt = 0;
  double2 *d_EB = nullptr;
  long long *d_offq = nullptr;
  double2 *d_EBcv = nullptr;       // sparse copies of d_EB
  unsigned char *d_EBci = nullptr;
  long long nEB = 0;
  int *d_bquart[2] = {nullptr, nullptr};
  long long nbquart[2] = {0, 0};
  int bquart_ilev = -1;
  std::vector<double> bqbound;  // [pair] sqrt max |(ab|ab)| of the LS pair, Breit
  float2 *d_EBf = nullptr;      // FP32 copy of d_EB scaled by 2^(kexp lambda) (tensor cores)
  std::vector<long long> bseg[2];  // Breit lists: class / bound-decade segments
  std::vector<int> bsegkey[2];
  std::vector<Run> bruns[2];
  bool btuned = false;
  std::vector<TuneRow> tune_rec, btune_rec;  // the tuner's last records (Coulomb, Breit)
  double2 *d_BX = nullptr;
  long long launches = 0;
  std::string err;
  bool bad = false;
};

// Batched build over independent instances (one context each): shells,
// pair tables and E-coefficients of all instances concatenated on the
// device, quartet lists of every instance merged per component class and
// grouped by angular class, one kernel launch per class for all instances.
struct bg_batch {
  int dev = -1;  // device of its instances
  int n = 0, ncomp = 1, hmlt = 0, isym = 0, racah1 = 1, prec = BG_PREC_FP64;
  double err_budget = 1e-7;  // BG_PREC_AUTO: estimated energy error allowed per build (Eh)
  std::vector<bg_ctx *> shadow;  // host copies of the instances' shells, bounds and rules
  std::vector<int> sbase;        // first batch shell of each instance
  std::vector<int> ndim;
  std::vector<Inst> inst;
  long long span = 0;            // complex elements the placement covers
  Shell *d_sh = nullptr;
  PairE *d_pe = nullptr;
  double2 *d_E = nullptr, *d_Ecv = nullptr;
  unsigned char *d_Eci = nullptr;
  float4 *d_Edf = nullptr, *d_Ddf = nullptr;
  double *d_qp = nullptr;  // k_qprep records of tensor-core launches (QP_CHUNK of them)
  float2 *d_Ef = nullptr;
  Inst *d_inst = nullptr;
  int *d_ndim = nullptr;
  int *d_quart[4] = {nullptr, nullptr, nullptr, nullptr};
  long long nquart[4] = {0, 0, 0, 0};
  int quart_ilev = -1;
  std::vector<long long> seg[4];  // BG_PREC_AUTO, as in bg_ctx
  std::vector<int> segkey[4];
  std::vector<Run> runs[4];
  bool tuned = false;
  long long launches = 0;
  std::string err;
  bool bad = false;
};

namespace {
std::string g_init_err;

int cuda_fail(bg_ctx *c, cudaError_t e, const char *what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  if (c) {
    c->err = m;
    c->bad = true;
  } else {
    g_init_err = m;
  }
  return BG_ERR_CUDA;
}

#define CK(ctx, call)                                   \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
  } while (0)

inline int kappa_of(int ka) {
  if (ka == 1) return -1;
  return (ka % 2 == 0) ? ka / 2 : -(ka / 2) - 1;
}

// One-time set-up of a device, done with that device current and recorded
// per device ordinal: the __constant__ Hermite and reciprocal tables, the
// split path's Boys table, and the >48 KB dynamic shared-memory opt-in of
// every quartet kernel.  All of them are properties of a device (a context on
// a second device gets its own), and none may be issued inside a stream
// capture, so the launchers never touch them.
constexpr int MAXDEV = 64;
std::mutex g_dev_mu;
bool g_dev_ready[MAXDEV] = {false};

const char *device_setup(int dev) {
  std::lock_guard<std::mutex> lk(g_dev_mu);
  if (dev < 0 || dev >= MAXDEV) return "device ordinal out of range";
  if (g_dev_ready[dev]) return nullptr;
  signed char t[NTR], u[NTR], v[NTR];
  int n = 0;
  for (int L = 0; L <= MAXLAM; ++L)
    for (int a = 0; a <= L; ++a)
      for (int b = 0; b <= L - a; ++b) {
        t[n] = (signed char)a; u[n] = (signed char)b; v[n] = (signed char)(L - a - b);
        ++n;
      }
  if (cudaMemcpyToSymbol(c_t, t, sizeof(t)) != cudaSuccess ||
      cudaMemcpyToSymbol(c_u, u, sizeof(u)) != cudaSuccess ||
      cudaMemcpyToSymbol(c_v, v, sizeof(v)) != cudaSuccess)
    return "Hermite index table upload failed";
  double rinv[NRINV];
  for (int k = 0; k < NRINV; ++k) rinv[k] = 1.0 / double(2 * k + 1);
  if (cudaMemcpyToSymbol(c_rinv, rinv, sizeof(rinv)) != cudaSuccess)
    return "reciprocal table upload failed";
  k_boys_table<<<(NBGRID + 127) / 128, 128>>>();
  {
    std::vector<unsigned short> hx((size_t)NTE * NHS, 0);
    for (int nn = 0; nn < NTE; ++nn)
      for (int ss = 0; ss < NTE; ++ss)
        hx[(size_t)nn * NHS + ss] =
            (unsigned short)hidx(t[nn] + t[ss], u[nn] + u[ss], v[nn] + v[ss]);
    if (cudaMemcpyToSymbol(g_hx, hx.data(), sizeof(unsigned short) * hx.size()) != cudaSuccess)
      return "Hankel index table upload failed";
  }
  // the tensor-core kernels: the per-block opt-in limit less their static
  // shared memory (the launches never ask for more than g_tc_smem_max)
  int optin = 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return "shared-memory opt-in query failed";
  const void *tck[6] = {(const void *)k_quartet_tc<256, true>,
                        (const void *)k_quartet_tc<512, true>,
                        (const void *)k_quartet_tc<256, false>,
                        (const void *)k_quartet_tc<512, false>,
                        (const void *)k_breit_tc<256>, (const void *)k_breit_tc<512>};
  size_t stat = 0;
  for (const void *f : tck) {
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, f) != cudaSuccess) return "kernel attribute query failed";
    stat = std::max(stat, fa.sharedSizeBytes);
  }
  g_tc_smem_max = std::min(TC_SMEM_MAX, (size_t)optin - stat);
  for (const void *f : tck)
    if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)g_tc_smem_max) != cudaSuccess)
      return "tensor-core kernel shared-memory opt-in failed";
  if (cudaFuncSetAttribute(k_quartet, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)quartet_smem()) != cudaSuccess ||
      cudaFuncSetAttribute(k_quartet_df, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)quartet_smem_df_max()) != cudaSuccess ||
      cudaFuncSetAttribute(k_breit, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)breit_smem()) != cudaSuccess)
    return "quartet kernel shared-memory opt-in failed";
  if (cudaDeviceSynchronize() != cudaSuccess || cudaGetLastError() != cudaSuccess)
    return "Boys table kernel failed";
  g_dev_ready[dev] = true;
  return nullptr;
}

// Every context and batch remembers the device it was made on; calls made
// while another device is current are refused (BG_ERR_STATE).
int current_device() {
  int d = -1;
  if (cudaGetDevice(&d) != cudaSuccess) return -1;
  return d;
}

int wrong_device(bg_ctx *c) {
  int d = current_device();
  if (d == c->dev) return 0;
  c->err = "context was made on device " + std::to_string(c->dev) + ", device " +
           std::to_string(d) + " is current";
  return BG_ERR_STATE;
}

// Decades of the Schwarz bound Q_ab Q_cd that split an angular class into
// segments: >= 1e1, [1, 1e1), ..., < 1e-5 (everything in one segment when
// no bounds exist).
constexpr int NBND = 8;
inline int bound_bucket(double b, bool have) {
  if (!have || !(b > 0.0)) return 0;
  int e = (int)std::floor(std::log10(b));
  return std::min(NBND - 1, std::max(0, 1 - e));
}

// Ordered shell quartets of the multi-centre build for one component class,
// with CLMFAST's centre and stage rules (bertha-scf.f:11672-11677,
// 12045-12084) and the one-centre parity rule (:11753-11764), handed to
// sink(a, b, c, d) one by one.
// With `sym`, (ab|cd) = (cd|ab) is used: only pairs ab >= cd (pair index
// a*ns+b) are listed for LL|LL and SS|SS, LL|SS lists every ordered pair and
// SS|LL none; the kernels digest each listed quartet for both orders.  The
// spinor relation (ba|dc) = (ab|cd)* halves the lists once more: of a
// quartet and its image only one is listed, and for a Hermitian density the
// image's J and K contributions are the conjugate transposes of the listed
// quartet's, which k_herm_complete adds at the end (quartets equal to their
// own image are digested with weight 1/2).
// Quartets come out grouped by angular class (l_a,l_b,l_c,l_d), highest
// first, so neighbouring CTAs carry similar work.  With a Schwarz threshold
// quartets with Q_ab Q_cd below it are left out (SCHWARZ :37889, at the
// level of shell pairs); within a class the pairs are visited in order of
// decreasing bound, so the scan of cd pairs stops at the first one below
// threshold/Q_ab.
struct PairRec {
  int a, b;
  double q;
  long long idx;
};

void pair_lists(const bg_ctx *c, int t, bool scr, std::vector<PairRec> (&pl)[MAXLB + 1][MAXLB + 1]) {
  for (int a = 0; a < c->ns; ++a)
    for (int b = 0; b < c->ns; ++b) {
      long long idx = (long long)a * c->ns + b;
      pl[c->shells[a].l][c->shells[b].l].push_back(
          {a, b, c->qbound.empty() ? 1.0 : c->qbound[idx * 2 + t], idx});
    }
  if (scr)
    for (auto &row : pl)
      for (auto &v : row)
        std::stable_sort(v.begin(), v.end(),
                         [](const PairRec &x, const PairRec &y) { return x.q > y.q; });
}

template <class Sink>
void gen_quartets(const bg_ctx *c, int t1, int t2, int ilev, bool sym, Sink &&sink) {
  int itt = 1 + 2 * t1 + t2;
  if (sym && t1 == 1 && t2 == 0) return;
  bool scr = c->screen > 0.0 && !c->qbound.empty();
  std::vector<PairRec> pl1[MAXLB + 1][MAXLB + 1], pl2[MAXLB + 1][MAXLB + 1];
  pair_lists(c, t1, scr, pl1);
  if (t2 != t1) pair_lists(c, t2, scr, pl2);
  auto &P2 = (t2 != t1) ? pl2 : pl1;
  for (int la = MAXLB; la >= 0; --la)
  for (int lb = MAXLB; lb >= 0; --lb)
  for (int lc = MAXLB; lc >= 0; --lc)
  for (int ld = MAXLB; ld >= 0; --ld) {
    const std::vector<PairRec> &X = pl1[la][lb], &Y = P2[lc][ld];
    if (X.empty() || Y.empty()) continue;
    bool par = ((la + lb) & 1) != ((lc + ld) & 1);
    for (const PairRec &x : X) {
      if (scr && x.q * Y[0].q < c->screen) break;
      const Shell &A = c->shells[x.a], &B = c->shells[x.b];
      for (const PairRec &y : Y) {
        if (scr && x.q * y.q < c->screen) break;
        if (sym && t1 == t2 && x.idx < y.idx) continue;
        if (sym) {
          // (ba|dc) = (ab|cd)*: keep the lexicographic maximum of the
          // quartet's orbit, the pair indices of (ab|cd) against those of
          // (ba|dc) and, within one class, of (dc|ba)
          long long pb = (long long)x.b * c->ns + x.a, qb = (long long)y.b * c->ns + y.a;
          if (x.idx < pb || (x.idx == pb && y.idx < qb)) continue;
          if (t1 == t2 && (x.idx < qb || (x.idx == qb && y.idx < pb))) continue;
        }
        const Shell &C = c->shells[y.a], &D = c->shells[y.b];
        int mcnt = 1 + (B.cnt != A.cnt) + (C.cnt != A.cnt && C.cnt != B.cnt) +
                   (D.cnt != A.cnt && D.cnt != B.cnt && D.cnt != C.cnt);
        if (mcnt == 1 && c->racah1) continue;
        if (ilev == 1 && itt > 1 && mcnt != 1) continue;
        if (ilev == 2 && itt > 3 && mcnt != 1) continue;
        if (mcnt == 1 && par) continue;
        sink(x.a, x.b, y.a, y.b, x.q * y.q);
      }
    }
  }
}


int launch_quartets(bg_ctx *c, const int *d_q, long long nq, int t1, int t2,
                    const double2 *d_D, int ldd, double *d_GD, double *d_GX,
                    int ldf, cudaStream_t st, int sym, double *bound);

// Schwarz bounds Q(ab,T) = sqrt(max |(ab|ab)|) of every shell pair and
// component, from the FP64 quartet kernel in bound mode (CLMDIAG :38126).
int compute_bounds(bg_ctx *c, cudaStream_t st) {
  int ns = c->ns;
  std::vector<int> diag;
  for (int a = 0; a < ns; ++a)
    for (int b = 0; b < ns; ++b) { diag.push_back(a); diag.push_back(b); diag.push_back(a); diag.push_back(b); }
  long long np = (long long)ns * ns;
  int *d_q = nullptr;
  double *d_b = nullptr;
  CK(c, cudaMalloc(&d_q, sizeof(int) * diag.size()));
  CK(c, cudaMalloc(&d_b, sizeof(double) * np));
  CK(c, cudaMemcpyAsync(d_q, diag.data(), sizeof(int) * diag.size(), cudaMemcpyHostToDevice, st));
  c->qbound.assign(np * 2, 0.0);
  std::vector<double> hb(np);
  for (int t = 0; t < c->ncomp; ++t) {
    int rc = launch_quartets(c, d_q, np, t, t, nullptr, 0, nullptr, nullptr, 0, st, 0, d_b);
    if (rc) { cudaFree(d_q); cudaFree(d_b); return rc; }
    CK(c, cudaMemcpyAsync(hb.data(), d_b, sizeof(double) * np, cudaMemcpyDeviceToHost, st));
    CK(c, cudaStreamSynchronize(st));
    for (long long p = 0; p < np; ++p) c->qbound[p * 2 + t] = sqrt(hb[p]);
  }
  cudaFree(d_q);
  cudaFree(d_b);
  return 0;
}

int launch_quartets_df(bg_ctx *c, const int *d_q, long long nq, int t1, int t2,
                       const double2 *d_D, int ldd, double *d_GD, double *d_GX, int ldf,
                       cudaStream_t st, float4 *ddf, int sym = 0, bool convert = true) {
  if (nq <= 0) return 0;
  size_t smem = quartet_smem_df(sym ? 1 : 0);
  int n = c->ndim;
  // convert = false: ddf already holds this density (one conversion per build)
  if (convert) {
    k_dconv<<<1024, 256, 0, st>>>(d_D, ldd, n, ddf);
    c->launches++;
  }
  QArgsDF a;
  a.inst = nullptr;
  a.sh = c->d_sh; a.pe = c->d_pe; a.E = c->d_Edf; a.D = ddf; a.Eci = c->d_Eci;
  a.GD = d_GD; a.GX = d_GX; a.ns = c->ns; a.ldd = n; a.ldf = ldf;
  a.nskp = c->nskp; a.isym = c->isym; a.racah1 = c->racah1; a.sym = sym;
  long long grid = std::min<long long>(nq, 152LL * 128);
  k_quartet_df<<<(unsigned)grid, DFTHREADS, smem, st>>>(a, (const int4 *)d_q, nq, t1, t2);
  CK(c, cudaGetLastError());
  c->launches++;
  return 0;
}

// Device address of g_noalloc_density for the current device, looked up
// once per device with that device current (cudaGetSymbolAddress).
float4 *noalloc_scratch(bg_ctx *c, int *rc) {
  static float4 *addr[64] = {nullptr};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 64) {
    *rc = cuda_fail(c, e == cudaSuccess ? cudaErrorInvalidDevice : e, "cudaGetDevice");
    return nullptr;
  }
  if (!addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_density);
    if (e != cudaSuccess) {
      *rc = cuda_fail(c, e, "cudaGetSymbolAddress");
      return nullptr;
    }
    addr[dev] = (float4 *)p;
  }
  *rc = 0;
  return addr[dev];
}

int launch_quartets_fp64(bg_ctx *c, const int *d_q, long long nq, int t1, int t2,
                         const double2 *d_D, int ldd, double *d_GD, double *d_GX, int ldf,
                         cudaStream_t st, int sym, double *bound);

// Tensor-core launch over list entries whose classes need at most n1 (D1)
// and n2 (D2) TMEM columns (tcq::N1MAX, tcq::N2MAX cover every class).  The
// double-float density copy ddf is made here unless convert is false.
int launch_quartets_tc(bg_ctx *c, const int *d_q, long long nq, int t1, int t2,
                       const double2 *d_D, int ldd, double *d_GD, double *d_GX, int ldf,
                       cudaStream_t st, int sym, int n1, int n2) {
  if (nq <= 0) return 0;
  if (!c->d_qp) CK(c, cudaMalloc(&c->d_qp, sizeof(double) * QPW * QP_CHUNK));
  // explicit lists (sym 0) are digested once: FP32 shared accumulators;
  // Fock builds (sym 2) accumulate in FP64 so that repeated builds agree
  const bool f64 = sym != 0;
  TcGeom g = tc_geom(n1, n2, false, f64);
  tcq::Args a;
  a.sh = c->d_sh; a.pe = c->d_pe; a.E = c->d_Ef; a.D = d_D;
  a.GD = d_GD; a.GX = d_GX; a.ldd = ldd; a.ldf = ldf; a.nskp = c->nskp;
  a.isym = c->isym; a.racah1 = c->racah1; a.sym = sym; a.inst = nullptr; a.qp = c->d_qp;
  a.tmem_cols = g.cols; a.n1max = n1; a.n2max = n2; a.nbuf = g.nbuf;
  for (long long s0 = 0; s0 < nq; s0 += QP_CHUNK) {
    long long m = std::min(QP_CHUNK, nq - s0);
    const int4 *qq = (const int4 *)d_q + s0;
    k_qprep<<<(unsigned)std::min<long long>((m + 127) / 128, 152LL * 16), 128, 0, st>>>(
        c->d_sh, qq, m, 2 * t1 + 2 * t2, c->d_qp);
    long long grid = std::min<long long>(m, 152LL * g.ctas_per_sm);
    if (g.nt == 512 && f64)
      k_quartet_tc<512, true><<<(unsigned)grid, 512, g.smem, st>>>(a, qq, m, t1, t2);
    else if (g.nt == 512)
      k_quartet_tc<512, false><<<(unsigned)grid, 512, g.smem, st>>>(a, qq, m, t1, t2);
    else if (f64)
      k_quartet_tc<256, true><<<(unsigned)grid, 256, g.smem, st>>>(a, qq, m, t1, t2);
    else
      k_quartet_tc<256, false><<<(unsigned)grid, 256, g.smem, st>>>(a, qq, m, t1, t2);
    CK(c, cudaGetLastError());
    c->launches += 2;
  }
  return 0;
}

// FP64, split-precision or tensor-core launch as the context's precision
// says (BG_PREC_AUTO takes the split kernel here: explicit and streamed
// lists are not tuned per class; the tensor-core kernel is sized for every
// class); bound mode is always FP64.
int launch_quartets(bg_ctx *c, const int *d_q, long long nq, int t1, int t2,
                    const double2 *d_D, int ldd, double *d_GD, double *d_GX,
                    int ldf, cudaStream_t st, int sym = 0, double *bound = nullptr) {
  if (nq <= 0) return 0;
  if (c->prec == BG_PREC_TC32 && !bound)
    return launch_quartets_tc(c, d_q, nq, t1, t2, d_D, ldd, d_GD, d_GX, ldf, st, sym, tcq::N1MAX,
                              tcq::N2MAX);
  if (c->prec != BG_PREC_FP64 && !bound) {
    int n = c->ndim;
    if (!c->d_Ddf) CK(c, cudaMalloc(&c->d_Ddf, sizeof(float4) * (size_t)n * n));
    return launch_quartets_df(c, d_q, nq, t1, t2, d_D, ldd, d_GD, d_GX, ldf, st, c->d_Ddf, sym);
  }
  return launch_quartets_fp64(c, d_q, nq, t1, t2, d_D, ldd, d_GD, d_GX, ldf, st, sym, bound);
}

int launch_quartets_fp64(bg_ctx *c, const int *d_q, long long nq, int t1, int t2,
                         const double2 *d_D, int ldd, double *d_GD, double *d_GX, int ldf,
                         cudaStream_t st, int sym, double *bound) {
  if (nq <= 0) return 0;
  size_t smem = quartet_smem();
  QArgs a;
  a.inst = nullptr;
  a.sh = c->d_sh; a.pe = c->d_pe; a.E = c->d_E; a.D = d_D;
  a.Ecv = c->d_Ecv; a.Eci = c->d_Eci;
  a.GD = d_GD; a.GX = d_GX; a.ns = c->ns; a.ldd = ldd; a.ldf = ldf;
  a.nskp = c->nskp; a.isym = c->isym; a.racah1 = c->racah1; a.sym = sym;
  a.bound = bound;
  long long grid = std::min<long long>(nq, 152LL * 64);
  k_quartet<<<(unsigned)grid, QT64, smem, st>>>(a, (const int4 *)d_q, nq, t1, t2);
  CK(c, cudaGetLastError());
  c->launches++;
  return 0;
}

// Sparse copies (k_ecompact) of an E array made of blocks of nt coefficients
// at the offsets given.
int compact_e(bg_ctx *c, const double2 *E, long long n, const std::vector<long long> &boff,
              const std::vector<int> &bnt, double2 **cv, unsigned char **ci) {
  CK(c, cudaMalloc(cv, sizeof(double2) * std::max<long long>(n, 1)));
  CK(c, cudaMalloc(ci, std::max<long long>(n, 1)));
  long long nb = (long long)boff.size();
  if (nb == 0) return 0;
  long long *d_off = nullptr;
  int *d_nt = nullptr;
  CK(c, cudaMalloc(&d_off, sizeof(long long) * nb));
  CK(c, cudaMalloc(&d_nt, sizeof(int) * nb));
  CK(c, cudaMemcpy(d_off, boff.data(), sizeof(long long) * nb, cudaMemcpyHostToDevice));
  CK(c, cudaMemcpy(d_nt, bnt.data(), sizeof(int) * nb, cudaMemcpyHostToDevice));
  k_ecompact<<<(unsigned)((nb + 127) / 128), 128>>>(E, *cv, *ci, nb, d_off, d_nt);
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaGetLastError();
  cudaFree(d_off);
  cudaFree(d_nt);
  if (e != cudaSuccess) return cuda_fail(c, e, "k_ecompact");
  return 0;
}

// sigma-coupled LS/SL E-coefficients of every ordered shell pair (the
// EILS/EISL lists of EQSAVE, bertha-scf.f:33644), generated once per context.
int breit_prepare(bg_ctx *c) {
  if (c->d_EB) return 0;
  int ns = c->ns;
  std::vector<long long> offq((size_t)ns * ns * 2), wstart((size_t)ns * ns * 2 + 1);
  long long off = 0, work = 0;
  for (int a = 0; a < ns; ++a)
    for (int b = 0; b < ns; ++b) {
      int la = c->shells[a].l, lb = c->shells[b].l;
      int nl = (2 * la + 1) * (2 * lb + 1);
      for (int comp = 0; comp < 2; ++comp) {
        size_t k = ((size_t)a * ns + b) * 2 + comp;
        offq[k] = off;
        off += (long long)nl * 6 * ntuv(la + lb + 1);
        wstart[k] = work;
        work += (long long)nl * 6;
      }
    }
  wstart[(size_t)ns * ns * 2] = work;
  long long *d_ws = nullptr;
  CK(c, cudaMalloc(&c->d_EB, sizeof(double2) * std::max<long long>(off, 1)));
  CK(c, cudaMalloc(&c->d_offq, sizeof(long long) * offq.size()));
  CK(c, cudaMalloc(&d_ws, sizeof(long long) * wstart.size()));
  CK(c, cudaMemcpy(c->d_offq, offq.data(), sizeof(long long) * offq.size(), cudaMemcpyHostToDevice));
  CK(c, cudaMemcpy(d_ws, wstart.data(), sizeof(long long) * wstart.size(), cudaMemcpyHostToDevice));
  if (work > 0) k_eqgen_q<<<(unsigned)((work + 63) / 64), 64>>>(c->d_sh, ns, c->d_offq, c->d_EB, work, d_ws);
  cudaError_t e = cudaDeviceSynchronize();
  cudaFree(d_ws);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(c, e, "k_eqgen_q");
  c->nEB = off;
  std::vector<long long> boff;
  std::vector<int> bnt;
  for (int a = 0; a < ns; ++a)
    for (int b = 0; b < ns; ++b) {
      int la = c->shells[a].l, lb = c->shells[b].l, nt = ntuv(la + lb + 1);
      int nblk = (2 * la + 1) * (2 * lb + 1) * 6;
      for (int comp = 0; comp < 2; ++comp)
        for (int k = 0; k < nblk; ++k) {
          boff.push_back(offq[((size_t)a * ns + b) * 2 + comp] + (long long)k * nt);
          bnt.push_back(nt);
        }
    }
  int rc = compact_e(c, c->d_EB, off, boff, bnt, &c->d_EBcv, &c->d_EBci);
  if (rc) return rc;
  // FP32 copy for the tensor-core kernel, scaled per pair like the
  // double-float Coulomb copy (2^(kexp lambda), kexp of the pair's exponent sum)
  CK(c, cudaMalloc(&c->d_EBf, sizeof(float2) * std::max<long long>(off, 1)));
  k_ebf<<<(unsigned)((long long)ns * ns * 2), 128>>>(c->d_EB, c->d_EBf, c->d_offq, c->d_pe,
                                                     c->d_sh, ns);
  cudaError_t e2 = cudaDeviceSynchronize();
  if (e2 == cudaSuccess) e2 = cudaGetLastError();
  if (e2 != cudaSuccess) return cuda_fail(c, e2, "k_ebf");
  return 0;
}

// Shell quartets of the Breit classes with BRTFAST's centre and stage rules
// (bertha-scf.f:17226-17231) and the one-centre parity rule (:17319-17329).
// With a Schwarz threshold, quartets with Q_ab Q_cd below it are left out:
// the Breit kernel -1/2 (delta_ij/r + r_i r_j/r^3) is negative semidefinite
// (its Fourier transform is -(4 pi/k^2)(delta_ij - k_i k_j/k^2)), so
// |(ab|cd)| <= Q_ab Q_cd with Q^2 the largest |(ab|ab)| over labels and
// m-signs (the Kramers partner of a density is its conjugate up to sign);
// the SL pair cd has the bound of the LS pair dc ((ab|cd)* = (ba|dc)).
// t2 = 0: (LS|LS), pairs ab >= cd only, each digested for both orders;
// t2 = 1: (LS|SL), digested for both orders, which covers the (SL|LS)
// class; of a quartet and its image (dc|ba) = (ab|cd)* only one is listed,
// the LL and SS blocks it feeds being completed as Hermitian matrices
// afterwards (Hermitian density).  The (SL|SL) class only feeds the SL
// block, which BRTFAST overwrites by conjugation of the LS block.
std::vector<int> build_breit_quartets(const bg_ctx *c, int t2, int ilev,
                                      std::vector<long long> *seg = nullptr,
                                      std::vector<int> *segkey = nullptr) {
  std::vector<int> out;
  bool scr = c->screen > 0.0 && !c->bqbound.empty();
  bool bnds = !c->bqbound.empty();
  std::vector<int> byl[MAXLB + 1];
  for (int s = 0; s < c->ns; ++s) byl[c->shells[s].l].push_back(s);
  if (seg) { seg->clear(); segkey->clear(); }
  std::vector<int> cls[NBND];
  for (int la = MAXLB; la >= 0; --la)
  for (int lb = MAXLB; lb >= 0; --lb)
  for (int lc = MAXLB; lc >= 0; --lc)
  for (int ld = MAXLB; ld >= 0; --ld) {
    for (int a : byl[la])
    for (int b : byl[lb])
      for (int cc : byl[lc])
      for (int d : byl[ld]) {
        long long pab = (long long)a * c->ns + b, pcd = (long long)cc * c->ns + d;
        if (t2 == 0 && pab < pcd) continue;
        if (t2 == 1) {
          // (dc|ba) = (ab|cd)* within (LS|SL): keep the larger of the two
          long long pdc = (long long)d * c->ns + cc, pba = (long long)b * c->ns + a;
          if (pab < pdc || (pab == pdc && pcd < pba)) continue;
        }
        int s4[4] = {c->shells[a].cnt, c->shells[b].cnt, c->shells[cc].cnt, c->shells[d].cnt};
        std::sort(s4, s4 + 4);
        int mcnt = 1;
        for (int k = 1; k < 4; ++k) mcnt += s4[k] != s4[k - 1];
        if (mcnt == 1 && c->racah1) continue;
        if (mcnt != 1 && ilev < 3) continue;
        if (mcnt == 1 && ((la + lb) & 1) != ((lc + ld) & 1)) continue;
        // Schwarz: Q(LS pair ab) Q(cd as LS pair for t2 = 0, dc for SL)
        double bnd = bnds ? c->bqbound[pab] *
                                c->bqbound[t2 == 0 ? pcd : (long long)d * c->ns + cc]
                          : 1.0;
        if (scr && bnd < c->screen) continue;
        std::vector<int> &v = cls[bound_bucket(bnd, bnds)];
        v.push_back(a); v.push_back(b); v.push_back(cc); v.push_back(d);
      }
    // this class's quartets, largest bound decade first
    for (int bk = 0; bk < NBND; ++bk) {
      if (cls[bk].empty()) continue;
      if (seg) {
        seg->push_back((long long)out.size() / 4);
        segkey->push_back(((la * 4 + lb) * 4 + lc) * 4 + ld);
      }
      out.insert(out.end(), cls[bk].begin(), cls[bk].end());
      cls[bk].clear();
    }
  }
  if (seg) seg->push_back((long long)out.size() / 4);
  return out;
}

int launch_breit(bg_ctx *c, const int *d_q, long long nq, int t1, int t2, const double2 *d_D,
                 int ldd, double *d_BX, int ldf, cudaStream_t st, int dual,
                 double *bound = nullptr) {
  if (nq <= 0) return 0;
  size_t smem = breit_smem();
  BArgs a;
  a.sh = c->d_sh; a.offq = c->d_offq; a.E = c->d_EB; a.D = d_D; a.BX = d_BX;
  a.Ecv = c->d_EBcv; a.Eci = c->d_EBci;
  a.ns = c->ns; a.ldd = ldd; a.ldf = ldf; a.nskp = c->nskp; a.isym = c->isym;
  a.racah1 = c->racah1; a.gaunt = c->gaunt; a.dual = dual; a.bound = bound;
  long long grid = std::min<long long>(nq, 152LL * 64);
  k_breit<<<(unsigned)grid, QT64, smem, st>>>(a, (const int4 *)d_q, nq, t1, t2);
  CK(c, cudaGetLastError());
  c->launches++;
  return 0;
}

// Tensor-core Breit launch over list entries whose classes need at most
// n1 + n2 TMEM columns; D is the FP64 density (leading dimension ldd).
int launch_breit_tc(bg_ctx *c, const int *d_q, long long nq, int t1, int t2, const double2 *D,
                    int ldd, double *d_BX, int ldf, cudaStream_t st, int dual, int n1, int n2) {
  if (nq <= 0) return 0;
  if (!c->d_qp) CK(c, cudaMalloc(&c->d_qp, sizeof(double) * QPW * QP_CHUNK));
  TcGeom g = tc_geom(n1, n2, true);
  tcq::ArgsB a;
  a.sh = c->d_sh; a.pe = c->d_pe; a.offq = c->d_offq; a.E = c->d_EBf; a.D = D; a.BX = d_BX;
  a.ns = c->ns; a.ldd = ldd; a.ldf = ldf; a.nskp = c->nskp; a.isym = c->isym;
  a.racah1 = c->racah1; a.gaunt = c->gaunt; a.dual = dual; a.qp = c->d_qp;
  a.tmem_cols = g.cols; a.n1max = n1; a.n2max = n2; a.nbuf = g.nbuf; a.tri = g.tri;
  // R to order la+lb+lc+ld+2, +2 more for the gauge term's derivatives
  int lextra = 2 + (c->gaunt ? 0 : 2);
  for (long long s0 = 0; s0 < nq; s0 += QP_CHUNK) {
    long long m = std::min(QP_CHUNK, nq - s0);
    const int4 *qq = (const int4 *)d_q + s0;
    k_qprep<<<(unsigned)std::min<long long>((m + 127) / 128, 152LL * 16), 128, 0, st>>>(
        c->d_sh, qq, m, lextra, c->d_qp);
    long long grid = std::min<long long>(m, 152LL * g.ctas_per_sm);
    if (g.nt == 512)
      k_breit_tc<512><<<(unsigned)grid, 512, g.smem, st>>>(a, qq, m, t1, t2);
    else
      k_breit_tc<256><<<(unsigned)grid, 256, g.smem, st>>>(a, qq, m, t1, t2);
    CK(c, cudaGetLastError());
    c->launches += 2;
  }
  return 0;
}

// Schwarz bounds of the LS pairs for the Breit build: k_breit in bound mode
// over the diagonal quartets (ab|ab) of the (LS|LS) class.
int compute_breit_bounds(bg_ctx *c, cudaStream_t st) {
  int ns = c->ns;
  std::vector<int> diag;
  for (int a = 0; a < ns; ++a)
    for (int b = 0; b < ns; ++b) { diag.push_back(a); diag.push_back(b); diag.push_back(a); diag.push_back(b); }
  long long np = (long long)ns * ns;
  int *d_q = nullptr;
  double *d_b = nullptr;
  CK(c, cudaMalloc(&d_q, sizeof(int) * diag.size()));
  CK(c, cudaMalloc(&d_b, sizeof(double) * np));
  CK(c, cudaMemcpyAsync(d_q, diag.data(), sizeof(int) * diag.size(), cudaMemcpyHostToDevice, st));
  int rc = launch_breit(c, d_q, np, 0, 0, nullptr, 0, nullptr, 0, st, 0, d_b);
  if (rc) { cudaFree(d_q); cudaFree(d_b); return rc; }
  std::vector<double> hb(np);
  CK(c, cudaMemcpyAsync(hb.data(), d_b, sizeof(double) * np, cudaMemcpyDeviceToHost, st));
  CK(c, cudaStreamSynchronize(st));
  c->bqbound.resize(np);
  for (long long p = 0; p < np; ++p) c->bqbound[p] = sqrt(hb[p]);
  cudaFree(d_q);
  cudaFree(d_b);
  return 0;
}

// Quartets kept as cached device lists per context at most; above this the
// lists are streamed (regenerated on the host every build, CHUNK_Q at a
// time, overlapping the kernels of the previous chunk).
constexpr long long CACHE_Q = 1LL << 28;  // 268M quartets, 4.3 GB (default)

constexpr long long CHUNK_Q = 1LL << 23;  // 8M quartets, 128 MB per buffer (default)

// Autotuner of BG_PREC_AUTO.  A list sorted by angular class has segments
// seg[i]..seg[i+1] of one class (l_a,l_b,l_c,l_d) each.  For every segment
// of at least TUNE_MIN quartets, each candidate kernel (FP64, the
// double-float split path, the 3xTF32 tensor-core path) digests the first
// min(size, TUNE_SAMPLE) quartets into zeroed scratch outputs; its energy
// terms sum_ij Re D_ij G_ij (J and K) are compared with the FP64 kernel's,
// and a second, event-timed run gives its time.  The sample's energy error
// scaled by size/sample (a bound for errors of random sign) estimates the
// segment's error.  Every segment first takes the faster of the two kernels
// with FP64-level accuracy (FP64, split); then segments switch to the
// tensor-core kernel in order of time saved per unit of estimated error
// while the summed estimates stay within the error budget (Eh).  Smaller
// segments take the FP64 kernel (launch- and latency-bound either way).
// Neighbouring segments with the same choice merge into one run (tensor-core
// runs only when they share a TMEM allocation size).
// launch(kind, start, count, n1, n2) issues one kernel over list entries
// [start, start + count); energy(eJ, eK) reduces the scratch outputs.
constexpr long long TUNE_MIN = 2048, TUNE_SAMPLE = 16384;

struct SegDims {
  int n1, n2;
};

SegDims seg_dims(int key, int t1, int t2) {
  int la = (key >> 6) & 3, lb = (key >> 4) & 3, lc = (key >> 2) & 3, ld = key & 3;
  SegDims d;
  bool swp;
  tcq::tc_dims(la, lb, lc, ld, t1, t2, d.n1, d.n2, swp);
  return d;
}

int g_gaunt_dims = 0;  // set by the Breit tuner: Gaunt-only kernel tables

SegDims seg_dims_breit(int key) {
  int la = (key >> 6) & 3, lb = (key >> 4) & 3, lc = (key >> 2) & 3, ld = key & 3;
  SegDims d;
  bool swp;
  tcq::tcb_dims(la, lb, lc, ld, g_gaunt_dims, d.n1, d.n2, swp);
  return d;
}

// Runs of one kernel kind over all segments (BG_PREC_TC32 on cached lists:
// tensor-core runs sized per class).
std::vector<Run> uniform_runs(const std::vector<long long> &seg, const std::vector<int> &key,
                              int t1, int t2, int kind, bool breit = false) {
  std::vector<Run> runs;
  for (size_t i = 0; i + 1 < seg.size(); ++i) {
    long long n = seg[i + 1] - seg[i];
    if (n <= 0) continue;
    SegDims d = breit ? seg_dims_breit(key[i]) : seg_dims(key[i], t1, t2);
    if (!runs.empty() && runs.back().start + runs.back().count == seg[i] &&
        (kind != KIND_TC || tc_geom(d.n1, d.n2, breit).cols ==
                                tc_geom(runs.back().n1, runs.back().n2, breit).cols)) {
      runs.back().count += n;
      runs.back().n1 = std::max(runs.back().n1, d.n1);
      runs.back().n2 = std::max(runs.back().n2, d.n2);
    } else {
      runs.push_back({seg[i], n, kind, d.n1, d.n2});
    }
  }
  return runs;
}

struct SegTune {
  long long start, n;
  int n1, n2;
  float t[3];     // ms on the sample per kind (0: untimed)
  double err[3];  // estimated segment energy error per kind (Eh)
  int kind;
};

template <class Launch, class Zero, class Energy>
int tune_runs(const int *list, const std::vector<long long> &seg, const std::vector<int> &key,
              int t1, int t2, cudaStream_t st, double budget, Launch &&launch, Zero &&zero,
              Energy &&energy, std::vector<Run> &runs, bool breit = false,
              std::vector<TuneRow> *rec = nullptr) {
  runs.clear();
  if (seg.size() < 2) return 0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return -1;
  // a segment above TUNE_SAMPLE quartets is timed and checked on an evenly
  // strided sample of it (the list order within a segment follows the
  // shells, so its first quartets are not representative)
  int *samp = nullptr;
  if (cudaMalloc(&samp, sizeof(int4) * TUNE_SAMPLE) != cudaSuccess) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return -1;
  }
  int rc = 0;
  std::vector<SegTune> tv;
  for (size_t i = 0; i + 1 < seg.size() && !rc; ++i) {
    long long n = seg[i + 1] - seg[i];
    if (n <= 0) continue;
    SegDims d = breit ? seg_dims_breit(key[i]) : seg_dims(key[i], t1, t2);
    SegTune x = {seg[i], n, d.n1, d.n2, {0.f, 0.f, 0.f}, {0.0, 0.0, 0.0}, KIND_FP64};
    if (n >= TUNE_MIN) {
      long long m = std::min(n, TUNE_SAMPLE);
      const int *q = list + 4 * seg[i];
      if (m < n) {
        long long stride = n / m;
        if (cudaMemcpy2DAsync(samp, sizeof(int4), q, sizeof(int4) * stride, sizeof(int4), m,
                              cudaMemcpyDeviceToDevice, st) != cudaSuccess) {
          rc = -1;
          break;
        }
        q = samp;
      }
      double ej[3] = {0, 0, 0}, ek[3] = {0, 0, 0};
      for (int k = 0; k < 3 && !rc; ++k) {
        if (breit && k == KIND_DF32) continue;  // the Breit build has no split-precision kernel
        rc = zero();
        if (!rc) rc = launch(k, q, m, d.n1, d.n2);
        if (!rc) rc = energy(ej[k], ek[k]);
        if (rc) break;
        cudaEventRecord(e0, st);
        rc = launch(k, q, m, d.n1, d.n2);
        cudaEventRecord(e1, st);
        if (!rc && cudaEventSynchronize(e1) != cudaSuccess) rc = -1;
        if (!rc) cudaEventElapsedTime(&x.t[k], e0, e1);
      }
      for (int k = 0; k < 3; ++k)
        x.err[k] = (fabs(ej[k] - ej[0]) + fabs(ek[k] - ek[0])) * (double)n / (double)m;
      x.kind = (!breit && x.t[1] < x.t[0]) ? KIND_DF32 : KIND_FP64;
    }
    tv.push_back(x);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamSynchronize(st);
  cudaFree(samp);
  if (rc) return rc;
  // tensor-core switches by time saved per error, within the budget
  std::vector<int> cand;
  for (size_t i = 0; i < tv.size(); ++i)
    if (tv[i].n >= TUNE_MIN && tv[i].t[2] > 0.f && tv[i].t[2] < tv[i].t[tv[i].kind]) cand.push_back((int)i);
  auto gain = [&](int i) {
    const SegTune &x = tv[i];
    double saved = (x.t[x.kind] - x.t[2]) * (double)x.n / (double)std::min(x.n, TUNE_SAMPLE);
    return saved / (x.err[2] + 1e-300);
  };
  std::sort(cand.begin(), cand.end(), [&](int a, int b) { return gain(a) > gain(b); });
  double used = 0.0;
  for (int i : cand)
    if (used + tv[i].err[2] <= budget) {
      used += tv[i].err[2];
      tv[i].kind = KIND_TC;
    }
  if (rec)
    for (size_t i = 0, j = 0; i + 1 < seg.size(); ++i) {
      if (seg[i + 1] - seg[i] <= 0) continue;
      const SegTune &x = tv[j++];
      rec->push_back({2 * t1 + t2, key[i], x.start, x.n, {x.t[0], x.t[1], x.t[2]},
                      {x.err[0], x.err[1], x.err[2]}, x.kind});
    }
  for (const SegTune &x : tv) {
    if (!runs.empty() && runs.back().kind == x.kind &&
        runs.back().start + runs.back().count == x.start &&
        (x.kind != KIND_TC ||
         tc_geom(x.n1, x.n2, breit).cols == tc_geom(runs.back().n1, runs.back().n2, breit).cols)) {
      runs.back().count += x.n;
      runs.back().n1 = std::max(runs.back().n1, x.n1);
      runs.back().n2 = std::max(runs.back().n2, x.n2);
    } else {
      runs.push_back({x.start, x.n, x.kind, x.n1, x.n2});
    }
  }
  return 0;
}

// Reorders a cached quartet list so that the segments digested by one kind
// of launch (the FP64 kernel, the split kernel, or the tensor-core kernel
// at one launch shape: TMEM columns, CTAs per SM, threads) are contiguous, and rebuilds seg, key and runs over the
// new order.  A build then makes one launch per kind and shape instead
// of one per stretch of neighbouring segments with the same choice (each
// launch ends with a partly idle GPU).  The segments and the kernel chosen
// for each are unchanged.  Returns nonzero on a CUDA failure.
int regroup_list(int *&d_list, std::vector<long long> &seg, std::vector<int> &key,
                 std::vector<Run> &runs, int t1, int t2, bool breit, cudaStream_t st) {
  if (seg.size() < 2 || seg.front() != 0 || runs.size() < 2) return 0;
  // launch shape of the tensor-core kernel (runs merge only within one)
  auto shape = [&](int n1, int n2) {
    TcGeom g = tc_geom(n1, n2, breit);
    return ((g.cols * 4 + g.ctas_per_sm) * 1024 + g.nt) * 4 + g.nbuf * 2 + g.tri;
  };
  struct S {
    long long start, n;
    int key, kind, shp, n1, n2;  // shp: launch shape (tensor cores)
  };
  std::vector<S> ss;
  size_t r = 0;
  for (size_t i = 0; i + 1 < seg.size(); ++i) {
    long long n = seg[i + 1] - seg[i];
    if (n <= 0) continue;
    while (r < runs.size() && runs[r].start + runs[r].count <= seg[i]) ++r;
    if (r == runs.size() || runs[r].start > seg[i]) return 0;  // not covered: keep the order
    SegDims d = breit ? seg_dims_breit(key[i]) : seg_dims(key[i], t1, t2);
    int kind = runs[r].kind;
    ss.push_back({seg[i], n, key[i], kind, kind == KIND_TC ? shape(d.n1, d.n2) : 0, d.n1, d.n2});
  }
  std::vector<int> ord(ss.size());
  for (size_t i = 0; i < ord.size(); ++i) ord[i] = (int)i;
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) {
    const S &x = ss[a], &y = ss[b];
    if (x.kind != y.kind) return x.kind < y.kind;
    if (x.shp != y.shp) return x.shp < y.shp;
    return x.kind == KIND_TC && (x.n1 != y.n1 ? x.n1 < y.n1 : x.n2 < y.n2);
  });
  long long tot = seg.back();
  int *nl = nullptr;
  if (cudaMalloc(&nl, sizeof(int4) * (size_t)tot) != cudaSuccess) return -1;
  std::vector<long long> nseg;
  std::vector<int> nkey;
  std::vector<Run> nruns;
  long long pos = 0;
  for (int o : ord) {
    const S &x = ss[o];
    if (cudaMemcpyAsync(nl + 4 * pos, d_list + 4 * x.start, sizeof(int4) * (size_t)x.n,
                        cudaMemcpyDeviceToDevice, st) != cudaSuccess) {
      cudaFree(nl);
      return -1;
    }
    nseg.push_back(pos);
    nkey.push_back(x.key);
    Run *b = nruns.empty() ? nullptr : &nruns.back();
    if (b && b->kind == x.kind &&
        (x.kind != KIND_TC ||
         (shape(b->n1, b->n2) == x.shp &&
          shape(std::max(b->n1, x.n1), std::max(b->n2, x.n2)) == x.shp))) {
      b->count += x.n;
      b->n1 = std::max(b->n1, x.n1);
      b->n2 = std::max(b->n2, x.n2);
    } else {
      nruns.push_back({pos, x.n, x.kind, x.n1, x.n2});
    }
    pos += x.n;
  }
  nseg.push_back(pos);
  if (cudaStreamSynchronize(st) != cudaSuccess) {
    cudaFree(nl);
    return -1;
  }
  cudaFree(d_list);
  d_list = nl;
  seg.swap(nseg);
  key.swap(nkey);
  runs.swap(nruns);
  return 0;
}

// sum_ij Re(D_ij G_ij) over an n x n block (leading dimensions ldd, ldg) or,
// with inst, over every instance's block; added to *out.
__global__ void k_edot(const double2 *D, long long ldd, const double2 *G, long long ldg, int n,
                       const Inst *inst, const int *ndim, int ninst, double *out) {
  double acc = 0.0;
  for (int k = 0; k < ninst; ++k) {
    const double2 *Dk = D, *Gk = G;
    long long m = n, ld1 = ldd, ld2 = ldg;
    if (inst) {
      Dk = D + inst[k].off;
      Gk = G + inst[k].off;
      m = ndim[k];
      ld1 = ld2 = inst[k].ld;
    }
    for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < m * m;
         w += (long long)gridDim.x * blockDim.x) {
      long long i = w % m, j = w / m;
      double2 d = Dk[i + ld1 * j], g = Gk[i + ld2 * j];
      acc += d.x * g.x - d.y * g.y;
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, acc);
}

// Tunes the cached lists of a context (first BG_PREC_AUTO build after the
// lists were made), with scratch outputs of NDIM^2.
int tune_ctx(bg_ctx *c, const double2 *d_D, int ldd, cudaStream_t st) {
  int n = c->ndim;
  double *gd = nullptr, *gx = nullptr, *d_e = nullptr;
  CK(c, cudaMalloc(&gd, sizeof(double2) * (size_t)n * n));
  CK(c, cudaMalloc(&gx, sizeof(double2) * (size_t)n * n));
  CK(c, cudaMalloc(&d_e, sizeof(double) * 2));
  if (!c->d_Ddf) CK(c, cudaMalloc(&c->d_Ddf, sizeof(float4) * (size_t)n * n));
  k_dconv<<<1024, 256, 0, st>>>(d_D, ldd, n, c->d_Ddf);
  int rc = 0;
  auto zero = [&]() {
    if (cudaMemsetAsync(gd, 0, sizeof(double2) * (size_t)n * n, st) != cudaSuccess ||
        cudaMemsetAsync(gx, 0, sizeof(double2) * (size_t)n * n, st) != cudaSuccess)
      return -1;
    return 0;
  };
  auto energy = [&](double &ej, double &ek) {
    if (cudaMemsetAsync(d_e, 0, sizeof(double) * 2, st) != cudaSuccess) return -1;
    k_edot<<<256, 256, 0, st>>>(d_D, ldd, (const double2 *)gd, n, n, nullptr, nullptr, 1, d_e);
    k_edot<<<256, 256, 0, st>>>(d_D, ldd, (const double2 *)gx, n, n, nullptr, nullptr, 1, d_e + 1);
    double h[2];
    if (cudaMemcpyAsync(h, d_e, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return -1;
    ej = h[0];
    ek = h[1];
    return 0;
  };
  for (int t1 = 0; t1 < c->ncomp && !rc; ++t1)
    for (int t2 = 0; t2 < c->ncomp && !rc; ++t2) {
      int k = 2 * t1 + t2;
      const int *q = c->d_quart[k];
      // the budget is shared by the component classes
      double budget = c->err_budget / (c->ncomp * c->ncomp);
      if (k == 0) c->tune_rec.clear();
      rc = tune_runs(q, c->seg[k], c->segkey[k], t1, t2, st, budget,
                     [&](int kind, const int *qq, long long m, int n1, int n2) {
        if (kind == KIND_DF32)
          return launch_quartets_df(c, qq, m, t1, t2, d_D, ldd, gd, gx, n, st, c->d_Ddf, 2, false);
        if (kind == KIND_TC)
          return launch_quartets_tc(c, qq, m, t1, t2, d_D, ldd, gd, gx, n, st, 2, n1, n2);
        return launch_quartets_fp64(c, qq, m, t1, t2, d_D, ldd, gd, gx, n, st, 2, nullptr);
      }, zero, energy, c->runs[k], false, &c->tune_rec);
    }
  cudaFree(gd);
  cudaFree(gx);
  cudaFree(d_e);
  if (rc) return rc > 0 ? rc : cuda_fail(c, cudaGetLastError(), "autotuning");
  for (int t1 = 0; t1 < c->ncomp; ++t1)
    for (int t2 = 0; t2 < c->ncomp; ++t2) {
      int k = 2 * t1 + t2;
      if (regroup_list(c->d_quart[k], c->seg[k], c->segkey[k], c->runs[k], t1, t2, false, st))
        return cuda_fail(c, cudaGetLastError(), "list regrouping");
    }
  c->tuned = true;
  return 0;
}

int stream_class(bg_ctx *c, int t1, int t2, int ilev, const double2 *d_D, int ldd, double *d_GD,
                 double *d_GX, int ldf, cudaStream_t st) {
  long long chunk = c->chunk_q > 0 ? c->chunk_q : CHUNK_Q;
  if (!c->h_chunk[0]) {
    for (int k = 0; k < 2; ++k) {
      CK(c, cudaMallocHost(&c->h_chunk[k], sizeof(int4) * chunk));
      CK(c, cudaMalloc(&c->d_chunk[k], sizeof(int4) * chunk));
      CK(c, cudaEventCreateWithFlags(&c->chunk_ev[k], cudaEventDisableTiming));
    }
  }
  // both buffers may still be read by the previous class's last copies
  for (int k = 0; k < 2; ++k) {
    cudaError_t e = cudaEventSynchronize(c->chunk_ev[k]);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaEventSynchronize");
  }
  int cur = 0, rc = 0;
  long long fill = 0;
  auto flush = [&]() {
    if (!fill || rc) return;
    cudaError_t e = cudaMemcpyAsync(c->d_chunk[cur], c->h_chunk[cur], sizeof(int4) * fill,
                                    cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) { rc = cuda_fail(c, e, "cudaMemcpyAsync"); return; }
    rc = launch_quartets(c, c->d_chunk[cur], fill, t1, t2, d_D, ldd, d_GD, d_GX, ldf, st, 2);
    if (rc) return;
    cudaEventRecord(c->chunk_ev[cur], st);
    cur ^= 1;
    // the other buffer was last read by the chunk before: wait for it
    e = cudaEventSynchronize(c->chunk_ev[cur]);
    if (e != cudaSuccess) rc = cuda_fail(c, e, "cudaEventSynchronize");
    fill = 0;
  };
  gen_quartets(c, t1, t2, ilev, true, [&](int a, int b, int cc, int d, double) {
    if (rc) return;
    int *h = c->h_chunk[cur] + 4 * fill;
    h[0] = a; h[1] = b; h[2] = cc; h[3] = d;
    if (++fill == chunk) flush();
  });
  flush();
  return rc;
}


int batch_fail(bg_batch *b, cudaError_t e, const char *what) {
  b->err = std::string(what) + ": " + cudaGetErrorString(e);
  b->bad = true;
  return BG_ERR_CUDA;
}

#define BK(b, call)                                      \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return batch_fail(b, e_, #call); \
  } while (0)

// Quartet lists of a batch for one stage: every instance's lists (CLMFAST
// rules of that instance, its Schwarz screening) in batch shell numbering,
// merged per component class and grouped by angular class, highest first.
int batch_lists(bg_batch *b, int ilev) {
  for (int k = 0; k < 4; ++k) {
    if (b->d_quart[k]) cudaFree(b->d_quart[k]);
    b->d_quart[k] = nullptr;
    b->nquart[k] = 0;
  }
  constexpr int NKEY = (MAXLB + 1) * (MAXLB + 1) * (MAXLB + 1) * (MAXLB + 1);
  for (int t1 = 0; t1 < b->ncomp; ++t1)
    for (int t2 = 0; t2 < b->ncomp; ++t2) {
      std::vector<std::vector<int>> bucket(NKEY * NBND);
      for (int i = 0; i < b->n; ++i) {
        const bg_ctx *c = b->shadow[i];
        int s0 = b->sbase[i];
        gen_quartets(c, t1, t2, ilev, true, [&](int a, int bb, int cc, int d, double bnd) {
          int key = ((c->shells[a].l * (MAXLB + 1) + c->shells[bb].l) * (MAXLB + 1) +
                     c->shells[cc].l) * (MAXLB + 1) + c->shells[d].l;
          std::vector<int> &v = bucket[(NKEY - 1 - key) * NBND + bound_bucket(bnd, !c->qbound.empty())];
          v.push_back(a + s0); v.push_back(bb + s0); v.push_back(cc + s0); v.push_back(d + s0);
        });
      }
      size_t tot = 0;
      for (auto &v : bucket) tot += v.size();
      int k = 2 * t1 + t2;
      b->nquart[k] = (long long)tot / 4;
      b->seg[k].clear();
      b->segkey[k].clear();
      b->runs[k].clear();
      if (!tot) continue;
      BK(b, cudaMalloc(&b->d_quart[k], sizeof(int) * tot));
      size_t pos = 0;
      for (auto &v : bucket) {
        if (v.empty()) continue;
        b->seg[k].push_back((long long)pos / 4);  // one angular class and bound decade per bucket
        b->segkey[k].push_back(NKEY - 1 - (int)(&v - &bucket[0]) / NBND);
        BK(b, cudaMemcpy(b->d_quart[k] + pos, v.data(), sizeof(int) * v.size(),
                         cudaMemcpyHostToDevice));
        pos += v.size();
        std::vector<int>().swap(v);
      }
      b->seg[k].push_back(b->nquart[k]);
    }
  b->quart_ilev = ilev;
  b->tuned = false;
  return 0;
}

// One launch of the FP64, split-precision or tensor-core quartet kernel
// (KIND_*) over nq quartets of one component class of a batch (a stretch
// of its list, or a tuning sample), both orders of each listed quartet
// digested; n1, n2 size the tensor-core launch.
int batch_launch(bg_batch *b, int t1, int t2, int kind, const int4 *quart, long long nq,
                 const double2 *d_D, double *d_GD, double *d_GX, cudaStream_t st, int n1 = 0,
                 int n2 = 0) {
  if (nq <= 0) return 0;
  if (kind == KIND_DF32) {
    QArgsDF a;
    a.sh = b->d_sh; a.pe = b->d_pe; a.E = b->d_Edf; a.D = b->d_Ddf; a.Eci = b->d_Eci;
    a.GD = d_GD; a.GX = d_GX; a.ns = 0; a.ldd = 0; a.ldf = 0; a.nskp = 0;
    a.isym = b->isym; a.racah1 = b->racah1; a.sym = 2; a.inst = b->d_inst;
    long long grid = std::min<long long>(nq, 152LL * 128);
    k_quartet_df<<<(unsigned)grid, DFTHREADS, quartet_smem_df(1), st>>>(a, quart, nq, t1, t2);
  } else if (kind == KIND_TC) {
    if (!b->d_qp) BK(b, cudaMalloc(&b->d_qp, sizeof(double) * QPW * QP_CHUNK));
    TcGeom g = tc_geom(n1, n2);
    tcq::Args a;
    a.sh = b->d_sh; a.pe = b->d_pe; a.E = b->d_Ef; a.D = d_D;
    a.GD = d_GD; a.GX = d_GX; a.ldd = 0; a.ldf = 0; a.nskp = 0;
    a.isym = b->isym; a.racah1 = b->racah1; a.sym = 2; a.inst = b->d_inst; a.qp = b->d_qp;
    a.tmem_cols = g.cols; a.n1max = n1; a.n2max = n2; a.nbuf = g.nbuf;
    for (long long s0 = 0; s0 < nq; s0 += QP_CHUNK) {
      long long m = std::min(QP_CHUNK, nq - s0);
      k_qprep<<<(unsigned)std::min<long long>((m + 127) / 128, 152LL * 16), 128, 0, st>>>(
          b->d_sh, quart + s0, m, 2 * t1 + 2 * t2, b->d_qp);
      long long grid = std::min<long long>(m, 152LL * g.ctas_per_sm);
      if (g.nt == 512)
        k_quartet_tc<512, true><<<(unsigned)grid, 512, g.smem, st>>>(a, quart + s0, m, t1, t2);
      else
        k_quartet_tc<256, true><<<(unsigned)grid, 256, g.smem, st>>>(a, quart + s0, m, t1, t2);
      b->launches += 2;
    }
    b->launches--;  // counted once more below
  } else {
    QArgs a;
    a.sh = b->d_sh; a.pe = b->d_pe; a.E = b->d_E; a.D = d_D; a.Ecv = b->d_Ecv; a.Eci = b->d_Eci;
    a.GD = d_GD; a.GX = d_GX; a.ns = 0; a.ldd = 0; a.ldf = 0; a.nskp = 0;
    a.isym = b->isym; a.racah1 = b->racah1; a.sym = 2; a.bound = nullptr; a.inst = b->d_inst;
    long long grid = std::min<long long>(nq, 152LL * 64);
    k_quartet<<<(unsigned)grid, QT64, quartet_smem(), st>>>(a, quart, nq, t1, t2);
  }
  BK(b, cudaGetLastError());
  b->launches++;
  return 0;
}

}  // namespace

extern "C" {

int bertha_gpu_init(bg_ctx **out, int ncnt, const double *bxyz, const int *nkap,
                    const int *nfnc, int mel, const double *bexl, int mbs, int hmlt,
                    int shape, int flags) {
  if (!out) return BG_ERR_ARG;
  *out = nullptr;
  if (ncnt < 1 || !bxyz || !nkap || !nfnc || !bexl || mel < 0 || mbs < 1) {
    g_init_err = "invalid argument";
    return BG_ERR_ARG;
  }
  if (hmlt < BG_HMLT_NORL || hmlt > BG_HMLT_DHFQ || shape < 0 || shape > 2) {
    g_init_err = "invalid hmlt or shape";
    return BG_ERR_ARG;
  }
  bg_ctx *c = new bg_ctx();
  c->ncnt = ncnt;
  c->cxyz.assign(bxyz, bxyz + 3 * ncnt);
  c->hmlt = hmlt;
  c->isym = shape;
  c->racah1 = (flags & BG_FLAG_NO_RACAH1) ? 0 : 1;
  c->gaunt = (flags & BG_FLAG_GAUNT) ? 1 : 0;
  c->ncomp = (hmlt == BG_HMLT_NORL) ? 1 : 2;
  c->lmax.resize(ncnt);
  int total = 0;
  for (int iz = 0; iz < ncnt; ++iz) {
    if (nkap[iz] < 1 || (nkap[iz] % 2) == 0) { g_init_err = "invalid NKAP"; delete c; return BG_ERR_ARG; }
    int lm = (nkap[iz] - 1) / 2;
    if (lm > MAXLB || lm > mel) { g_init_err = "LMAX beyond BG_MAX_L"; delete c; return BG_ERR_CAPACITY; }
    c->lmax[iz] = lm;
    for (int l = 0; l <= lm; ++l) {
      int n = nfnc[l + (mel + 1) * iz];
      if (n < 0 || n > mbs) { g_init_err = "invalid NFNC"; delete c; return BG_ERR_ARG; }
      total += 4 * (2 * l + 1) * n;
    }
  }
  c->ndim = hmlt == BG_HMLT_NORL ? total / 2 : total;
  c->nskp = hmlt == BG_HMLT_NORL ? 0 : total / 2;
  // FOCKIND layout (bertha-scf.f:2582-2648)
  const int NK = 2 * MAXLB + 2;
  c->lrge.assign((size_t)ncnt * NK * 28, -1);
  int ilst = 0;
  for (int iz = 0; iz < ncnt; ++iz)
    for (int imv = 0; imv <= MAXLB; ++imv) {
      int mqn = 2 * imv + 1;
      for (int sg = 0; sg < 2; ++sg)
        for (int ka = 1; ka <= nkap[iz]; ++ka) {
          int kq = kappa_of(ka);
          int nb = nfnc[lval(kq) + (mel + 1) * iz];
          if (2 * abs(kq) - 1 >= mqn) {
            c->lrge[((size_t)iz * NK + ka) * 28 + mqn - 1 + sg] = ilst;
            ilst += nb;
          }
        }
    }
  // shells in the order centre, l, exponent
  for (int iz = 0; iz < ncnt; ++iz)
    for (int l = 0; l <= c->lmax[iz]; ++l) {
      int n = nfnc[l + (mel + 1) * iz];
      for (int i = 0; i < n; ++i) {
        Shell s;
        memset(&s, 0, sizeof(s));
        s.x = bxyz[3 * iz]; s.y = bxyz[3 * iz + 1]; s.z = bxyz[3 * iz + 2];
        s.alpha = bexl[i + (size_t)mbs * (l + (size_t)(mel + 1) * iz)];
        if (!(s.alpha > 0.0)) { g_init_err = "non-positive exponent"; delete c; return BG_ERR_ARG; }
        s.l = l; s.cnt = iz; s.ibas = i;
        for (int lab = 0; lab < 2 * l + 1; ++lab) {
          int kq, ma;
          label_of(l, lab, kq, ma);
          int ka = (kq == -1) ? 1 : (kq > 0 ? 2 * kq : 2 * (-kq - 1) + 1);
          s.fock[lab][0] = c->lrge[((size_t)iz * NK + ka) * 28 + 2 * ma - 2] + i;
          s.fock[lab][1] = c->lrge[((size_t)iz * NK + ka) * 28 + 2 * ma - 1] + i;
        }
        c->shells.push_back(s);
      }
    }
  c->ns = (int)c->shells.size();
  for (int a = 0; a < c->ns; ++a) {
    c->shells[a].inst = 0;
    c->shells[a].prow = a * c->ns;
  }
  c->dev = current_device();
  if (const char *why = device_setup(c->dev)) {
    g_init_err = std::string("device set-up failed: ") + why + " (" +
                 cudaGetErrorString(cudaGetLastError()) + ")";
    delete c;
    return BG_ERR_CUDA;
  }
  // E-coefficient storage for every ordered shell pair and component
  int ns = c->ns, ncomp = c->ncomp;
  std::vector<PairE> pe((size_t)ns * ns);
  std::vector<long long> wstart((size_t)ns * ns * ncomp + 1);
  long long off = 0, work = 0;
  for (int a = 0; a < ns; ++a)
    for (int b = 0; b < ns; ++b) {
      PairE &p = pe[(size_t)a * ns + b];
      p.off[0] = p.off[1] = -1;
      p.kexp = half_floor_log2(2.0 * (c->shells[a].alpha + c->shells[b].alpha));
      p.pad = 0;
      int la = c->shells[a].l, lb = c->shells[b].l;
      int nl = (2 * la + 1) * (2 * lb + 1);
      for (int comp = 0; comp < ncomp; ++comp) {
        p.off[comp] = off;
        off += (long long)nl * 2 * ntuv(la + lb + 2 * comp);
        wstart[((size_t)a * ns + b) * ncomp + comp] = work;
        work += (long long)nl * 2;
      }
    }
  wstart[(size_t)ns * ns * ncomp] = work;
  c->nE = off;
  cudaError_t e;
  if ((e = cudaMalloc(&c->d_sh, sizeof(Shell) * ns)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_pe, sizeof(PairE) * pe.size())) != cudaSuccess ||
      (e = cudaMalloc(&c->d_E, sizeof(double2) * std::max<long long>(off, 1))) != cudaSuccess) {
    cuda_fail(nullptr, e, "cudaMalloc");
    bertha_gpu_free(c);
    return BG_ERR_CUDA;
  }
  long long *d_ws = nullptr;
  if ((e = cudaMalloc(&d_ws, sizeof(long long) * wstart.size())) != cudaSuccess) {
    cuda_fail(nullptr, e, "cudaMalloc");
    bertha_gpu_free(c);
    return BG_ERR_CUDA;
  }
  cudaMemcpy(c->d_sh, c->shells.data(), sizeof(Shell) * ns, cudaMemcpyHostToDevice);
  cudaMemcpy(c->d_pe, pe.data(), sizeof(PairE) * pe.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(d_ws, wstart.data(), sizeof(long long) * wstart.size(), cudaMemcpyHostToDevice);
  int thr = 64;
  if (work > 0) {
    k_eqgen<<<(unsigned)((work + thr - 1) / thr), thr>>>(c->d_sh, ns, c->d_pe, ncomp, c->d_E, work, d_ws);
  }
  e = cudaDeviceSynchronize();
  cudaFree(d_ws);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    cuda_fail(nullptr, e, "k_eqgen");
    bertha_gpu_free(c);
    return BG_ERR_CUDA;
  }
  // double-float copy for the split-precision path
  if ((e = cudaMalloc(&c->d_Edf, sizeof(float4) * std::max<long long>(off, 1))) != cudaSuccess) {
    cuda_fail(nullptr, e, "cudaMalloc");
    bertha_gpu_free(c);
    return BG_ERR_CUDA;
  }
  k_econv<<<(unsigned)((long long)ns * ns), 128>>>(c->d_E, c->d_Edf, c->d_pe, c->d_sh, ns, ncomp);
  if ((e = cudaMalloc(&c->d_Ef, sizeof(float2) * std::max<long long>(off, 1))) != cudaSuccess) {
    cuda_fail(nullptr, e, "cudaMalloc");
    bertha_gpu_free(c);
    return BG_ERR_CUDA;
  }
  k_ef<<<1024, 256>>>(c->d_Edf, c->d_Ef, off);
  e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    cuda_fail(nullptr, e, "k_econv");
    bertha_gpu_free(c);
    return BG_ERR_CUDA;
  }
  {
    std::vector<long long> boff;
    std::vector<int> bnt;
    for (int a = 0; a < ns; ++a)
      for (int b = 0; b < ns; ++b) {
        int la = c->shells[a].l, lb = c->shells[b].l;
        int nblk = (2 * la + 1) * (2 * lb + 1) * 2;
        for (int comp = 0; comp < ncomp; ++comp) {
          int nt = ntuv(la + lb + 2 * comp);
          for (int k = 0; k < nblk; ++k) {
            boff.push_back(pe[(size_t)a * ns + b].off[comp] + (long long)k * nt);
            bnt.push_back(nt);
          }
        }
      }
    if (compact_e(c, c->d_E, off, boff, bnt, &c->d_Ecv, &c->d_Eci)) {
      g_init_err = c->err;
      bertha_gpu_free(c);
      return BG_ERR_CUDA;
    }
  }
  *out = c;
  return BG_OK;
}

int bertha_gpu_set_screening(bg_ctx *c, double threshold) {
  if (!c || !(threshold >= 0.0)) return BG_ERR_ARG;
  if (threshold != c->screen) c->quart_ilev = c->bquart_ilev = -1;  // rebuild the lists
  c->screen = threshold;
  return BG_OK;
}

int bertha_gpu_set_precision(bg_ctx *c, int prec) {
  if (!c) return BG_ERR_ARG;
  if (prec != BG_PREC_FP64 && prec != BG_PREC_DF32 && prec != BG_PREC_AUTO &&
      prec != BG_PREC_TC32)
    return BG_ERR_ARG;
  if (prec != c->prec) c->tuned = c->btuned = false;
  c->prec = prec;
  return BG_OK;
}

int bertha_gpu_set_list_limits(bg_ctx *c, long long cache_quartets, long long chunk_quartets) {
  if (!c || cache_quartets < 0 || chunk_quartets < 0) return BG_ERR_ARG;
  if (c->h_chunk[0] && chunk_quartets != c->chunk_q) return BG_ERR_STATE;  // buffers exist
  c->cache_q = cache_quartets;
  c->chunk_q = chunk_quartets;
  c->quart_ilev = -1;
  return BG_OK;
}

int bertha_gpu_dims(const bg_ctx *c, int *ndim, int *nskp) {
  if (!c) return BG_ERR_ARG;
  if (ndim) *ndim = c->ndim;
  if (nskp) *nskp = c->nskp;
  return BG_OK;
}

int bertha_gpu_shells(const bg_ctx *c, int *nshell, int *cnt, int *l, int *ibas) {
  if (!c) return BG_ERR_ARG;
  if (nshell) *nshell = c->ns;
  for (int s = 0; s < c->ns; ++s) {
    if (cnt) cnt[s] = c->shells[s].cnt;
    if (l) l[s] = c->shells[s].l;
    if (ibas) ibas[s] = c->shells[s].ibas;
  }
  return BG_OK;
}

int bertha_gpu_layout(const bg_ctx *c, int *lrge) {
  if (!c || !lrge) return BG_ERR_ARG;
  memcpy(lrge, c->lrge.data(), sizeof(int) * c->lrge.size());
  return BG_OK;
}

long long bertha_gpu_launches(const bg_ctx *c) { return c ? c->launches : 0; }

namespace {
void auto_stats(const std::vector<Run> (&runs)[4], long long *nq, int *nr) {
  nq[0] = nq[1] = nq[2] = 0;
  int r = 0;
  for (int k = 0; k < 4; ++k)
    for (const Run &x : runs[k]) {
      nq[x.kind] += x.count;
      ++r;
    }
  if (nr) *nr = r;
}
}  // namespace

int bertha_gpu_auto_stats(const bg_ctx *c, long long *nq_fp64, long long *nq_df32, int *nruns) {
  if (!c) return BG_ERR_ARG;
  long long nq[3];
  auto_stats(c->runs, nq, nruns);
  if (nq_fp64) *nq_fp64 = nq[0];
  if (nq_df32) *nq_df32 = nq[1];
  return BG_OK;
}

int bertha_gpu_kernel_stats(const bg_ctx *c, long long *nq, int *nruns) {
  if (!c || !nq) return BG_ERR_ARG;
  auto_stats(c->runs, nq, nruns);
  return BG_OK;
}

int bertha_gpu_breit_kernel_stats(const bg_ctx *c, long long *nq, int *nruns) {
  if (!c || !nq) return BG_ERR_ARG;
  nq[0] = nq[1] = nq[2] = 0;
  int r = 0;
  for (int k = 0; k < 2; ++k)
    for (const Run &x : c->bruns[k]) {
      nq[x.kind] += x.count;
      ++r;
    }
  if (nruns) *nruns = r;
  return BG_OK;
}

int bertha_gpu_batch_auto_stats(const bg_batch *b, long long *nq_fp64, long long *nq_df32,
                                int *nruns) {
  if (!b) return BG_ERR_ARG;
  long long nq[3];
  auto_stats(b->runs, nq, nruns);
  if (nq_fp64) *nq_fp64 = nq[0];
  if (nq_df32) *nq_df32 = nq[1];
  return BG_OK;
}

int bertha_gpu_batch_kernel_stats(const bg_batch *b, long long *nq, int *nruns) {
  if (!b || !nq) return BG_ERR_ARG;
  auto_stats(b->runs, nq, nruns);
  return BG_OK;
}

int bertha_gpu_tuning_record(const bg_ctx *c, int breit, int cap, int *info,
                             double *vals, int *nrows) {
  if (!c || !nrows) return BG_ERR_ARG;
  const std::vector<TuneRow> &r = breit ? c->btune_rec : c->tune_rec;
  *nrows = (int)r.size();
  if (!info || !vals) return BG_OK;
  for (int i = 0; i < (int)r.size() && i < cap; ++i) {
    info[4 * i] = r[i].comp;
    info[4 * i + 1] = r[i].key;
    info[4 * i + 2] = (int)std::min<long long>(r[i].n, 0x7fffffff);
    info[4 * i + 3] = r[i].kind;
    for (int k = 0; k < 3; ++k) {
      vals[6 * i + k] = r[i].t[k];
      vals[6 * i + 3 + k] = r[i].err[k];
    }
  }
  return BG_OK;
}

int bertha_gpu_set_error_budget(bg_ctx *c, double eh) {
  if (!c || !(eh >= 0.0)) return BG_ERR_ARG;
  if (eh != c->err_budget) c->tuned = c->btuned = false;
  c->err_budget = eh;
  return BG_OK;
}

int bertha_gpu_batch_set_error_budget(bg_batch *b, double eh) {
  if (!b || !(eh >= 0.0)) return BG_ERR_ARG;
  if (eh != b->err_budget) b->tuned = false;
  b->err_budget = eh;
  return BG_OK;
}

int bertha_gpu_device_status(int *status) {
  if (!status) return BG_ERR_ARG;
  int v = 0;
  if (cudaDeviceSynchronize() != cudaSuccess) return BG_ERR_CUDA;
  if (cudaMemcpyFromSymbol(&v, tcq::g_tc_status, sizeof(int)) != cudaSuccess) return BG_ERR_CUDA;
  int z = 0;
  if (cudaMemcpyToSymbol(tcq::g_tc_status, &z, sizeof(int)) != cudaSuccess) return BG_ERR_CUDA;
  *status = v;
  return BG_OK;
}

const char *bertha_gpu_last_error(const bg_ctx *c) {
  return c ? c->err.c_str() : g_init_err.c_str();
}

int bertha_gpu_quartets(bg_ctx *c, const int *d_q, long long nq, int t1, int t2,
                        const double *d_dent, int ldd, double *d_gdir, double *d_gxch,
                        int ldf, void *stream) {
  if (!c) return BG_ERR_ARG;
  if (c->bad) return BG_ERR_STATE;
  if (int rd = wrong_device(c)) return rd;
  if (t1 < 0 || t1 >= c->ncomp || t2 < 0 || t2 >= c->ncomp || nq < 0 || ldd < c->ndim ||
      ldf < c->ndim || (nq > 0 && (!d_q || !d_dent || !d_gdir || !d_gxch)))
    return BG_ERR_ARG;
  c->launches = 0;
  return launch_quartets(c, d_q, nq, t1, t2, (const double2 *)d_dent, ldd, d_gdir, d_gxch,
                         ldf, (cudaStream_t)stream);
}

int bertha_gpu_quartets_segments(bg_ctx *c, const int *d_q, int nseg, const long long *seg,
                                 const int *lclass, int t1, int t2, const double *d_dent,
                                 int ldd, double *d_gdir, double *d_gxch, int ldf, void *stream) {
  if (!c) return BG_ERR_ARG;
  if (c->bad) return BG_ERR_STATE;
  if (int rd = wrong_device(c)) return rd;
  if (t1 < 0 || t1 >= c->ncomp || t2 < 0 || t2 >= c->ncomp || nseg < 0 || !seg || !lclass ||
      ldd < c->ndim || ldf < c->ndim)
    return BG_ERR_ARG;
  std::vector<long long> sv(seg, seg + nseg + 1);
  std::vector<int> keys(nseg);
  for (int i = 0; i < nseg; ++i) {
    if (sv[i] < 0 || sv[i + 1] < sv[i]) return BG_ERR_ARG;
    int key = 0;
    for (int j = 0; j < 4; ++j) {
      int l = lclass[4 * i + j];
      if (l < 0 || l > MAXLB) return BG_ERR_ARG;
      key = key * 4 + l;
    }
    keys[i] = key;
  }
  long long nq = nseg ? sv[nseg] - sv[0] : 0;
  if (nq > 0 && (!d_q || !d_dent || !d_gdir || !d_gxch)) return BG_ERR_ARG;
  c->launches = 0;
  if (nq <= 0) return BG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const double2 *D = (const double2 *)d_dent;
  if (c->prec != BG_PREC_TC32)
    return launch_quartets(c, d_q + 4 * sv[0], nq, t1, t2, D, ldd, d_gdir, d_gxch, ldf, st);
  // tensor cores: launches sized per class (runs of classes sharing a TMEM
  // allocation size), each reading the FP64 density
  for (const Run &r : uniform_runs(sv, keys, t1, t2, KIND_TC)) {
    int rc = launch_quartets_tc(c, d_q + 4 * r.start, r.count, t1, t2, D, ldd, d_gdir, d_gxch,
                                ldf, st, 0, r.n1, r.n2);
    if (rc) return rc;
  }
  return BG_OK;
}

int bertha_gpu_quartets_noalloc(bg_ctx *c, const int *d_q, long long nq, int t1, int t2,
                                const double *d_dent, int ldd, double *d_gdir,
                                double *d_gxch, int ldf, void *stream) {
  if (!c) return BG_ERR_ARG;
  if (c->bad) return BG_ERR_STATE;
  if (int rd = wrong_device(c)) return rd;
  if (t1 < 0 || t1 >= c->ncomp || t2 < 0 || t2 >= c->ncomp || nq < 0 || ldd < c->ndim ||
      ldf < c->ndim || (nq > 0 && (!d_q || !d_dent || !d_gdir || !d_gxch)))
    return BG_ERR_ARG;
  if (c->ndim > BG_NOALLOC_MAX_NDIM) {
    c->err = "bertha_gpu_quartets_noalloc: NDIM " + std::to_string(c->ndim) +
             " exceeds BG_NOALLOC_MAX_NDIM " + std::to_string(BG_NOALLOC_MAX_NDIM);
    return BG_ERR_CAPACITY;
  }
  int rc = 0;
  float4 *scratch = noalloc_scratch(c, &rc);
  if (!scratch) return rc;
  c->launches = 0;
  return launch_quartets_df(c, d_q, nq, t1, t2, (const double2 *)d_dent, ldd, d_gdir, d_gxch,
                            ldf, (cudaStream_t)stream, scratch);
}

int bertha_gpu_clmfast_device(bg_ctx *c, const double *d_dent, int ldd, int ilev,
                              double *d_gdir, double *d_gxch, int ldf, void *stream) {
  if (!c) return BG_ERR_ARG;
  if (c->bad) return BG_ERR_STATE;
  if (int rd = wrong_device(c)) return rd;
  if (ilev < 1 || ilev > 4 || ldd < c->ndim || ldf < c->ndim) return BG_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  c->launches = 0;
  if (c->hmlt == BG_HMLT_BARE) return BG_OK;  // CLMFAST returns at once (:11579)
  k_zero2d<<<1024, 256, 0, st>>>(d_gdir, c->ndim, ldf);
  k_zero2d<<<1024, 256, 0, st>>>(d_gxch, c->ndim, ldf);
  CK(c, cudaGetLastError());
  c->launches += 2;
  // bounds for screening and, under BG_PREC_AUTO, for the bound decades
  if ((c->screen > 0.0 || c->prec == BG_PREC_AUTO) && c->qbound.empty()) {
    int rc = compute_bounds(c, st);
    if (rc) return rc;
    c->quart_ilev = -1;
  }
  if (c->quart_ilev != ilev) {
    for (int k = 0; k < 4; ++k) {
      if (c->d_quart[k]) cudaFree(c->d_quart[k]);
      c->d_quart[k] = nullptr;
      c->nquart[k] = 0;
    }
    c->stream_lists = false;
    long long total = 0;
    std::vector<int> q[4];
    // each angular class's quartets grouped by the decade of their Schwarz
    // bound (largest first): segments of one class and bound decade, so that
    // the autotuner can give the small-magnitude part of a class another
    // kernel than its large part
    bool bnds = !c->qbound.empty();
    for (int t1 = 0; t1 < c->ncomp && !c->stream_lists; ++t1)
      for (int t2 = 0; t2 < c->ncomp && !c->stream_lists; ++t2) {
        int k = 2 * t1 + t2;
        std::vector<int> cls[NBND];
        int curkey = -1;
        c->seg[k].clear();
        c->segkey[k].clear();
        auto flush = [&]() {
          for (int bk = 0; bk < NBND; ++bk) {
            if (cls[bk].empty()) continue;
            c->seg[k].push_back((long long)q[k].size() / 4);
            c->segkey[k].push_back(curkey);
            q[k].insert(q[k].end(), cls[bk].begin(), cls[bk].end());
            cls[bk].clear();
          }
        };
        gen_quartets(c, t1, t2, ilev, true, [&](int a, int b, int cc, int d, double bnd) {
          if (c->stream_lists) return;
          int key = ((c->shells[a].l * 4 + c->shells[b].l) * 4 + c->shells[cc].l) * 4 +
                    c->shells[d].l;
          if (key != curkey) {
            flush();
            curkey = key;
          }
          std::vector<int> &v = cls[bound_bucket(bnd, bnds)];
          v.push_back(a); v.push_back(b); v.push_back(cc); v.push_back(d);
          if (++total > (c->cache_q > 0 ? c->cache_q : CACHE_Q)) c->stream_lists = true;
        });
        flush();
        c->seg[k].push_back((long long)q[k].size() / 4);
      }
    c->tuned = false;
    if (!c->stream_lists)
      for (int k = 0; k < 4; ++k) {
        c->runs[k].clear();
        c->nquart[k] = (long long)q[k].size() / 4;
        if (!q[k].empty()) {
          CK(c, cudaMalloc(&c->d_quart[k], sizeof(int) * q[k].size()));
          CK(c, cudaMemcpy(c->d_quart[k], q[k].data(), sizeof(int) * q[k].size(),
                           cudaMemcpyHostToDevice));
        }
      }
    c->quart_ilev = ilev;
  }
  // per-run kernels: tuned (BG_PREC_AUTO) or the tensor-core kernel sized
  // per class (BG_PREC_TC32) on cached lists
  bool byrun = (c->prec == BG_PREC_AUTO || c->prec == BG_PREC_TC32) && !c->stream_lists;
  if (byrun && !c->tuned) {
    if (c->prec == BG_PREC_AUTO) {
      int rc = tune_ctx(c, (const double2 *)d_dent, ldd, st);
      if (rc) return rc;
    } else {
      for (int t1 = 0; t1 < c->ncomp; ++t1)
        for (int t2 = 0; t2 < c->ncomp; ++t2) {
          int k = 2 * t1 + t2;
          c->runs[k] = uniform_runs(c->seg[k], c->segkey[k], t1, t2, KIND_TC);
          if (regroup_list(c->d_quart[k], c->seg[k], c->segkey[k], c->runs[k], t1, t2, false, st))
            return cuda_fail(c, cudaGetLastError(), "list regrouping");
        }
      c->tuned = true;
    }
  }
  if (byrun) {
    // one double-float copy of the density for all split-precision runs
    // (the tensor-core kernels read the FP64 density)
    bool any_f = false;
    for (int k = 0; k < 4; ++k)
      for (const Run &r : c->runs[k]) any_f |= r.kind == KIND_DF32;
    if (any_f) {
      if (!c->d_Ddf) CK(c, cudaMalloc(&c->d_Ddf, sizeof(float4) * (size_t)c->ndim * c->ndim));
      k_dconv<<<1024, 256, 0, st>>>((const double2 *)d_dent, ldd, c->ndim, c->d_Ddf);
      CK(c, cudaGetLastError());
      c->launches++;
    }
  }
  for (int t1 = c->ncomp - 1; t1 >= 0; --t1)
    for (int t2 = c->ncomp - 1; t2 >= 0; --t2) {
      int k = 2 * t1 + t2, rc = 0;
      if (c->stream_lists)
        rc = stream_class(c, t1, t2, ilev, (const double2 *)d_dent, ldd, d_gdir, d_gxch, ldf, st);
      else if (byrun)
        for (const Run &r : c->runs[k]) {
          const int *q = c->d_quart[k] + 4 * r.start;
          const double2 *D = (const double2 *)d_dent;
          if (r.kind == KIND_DF32)
            rc = launch_quartets_df(c, q, r.count, t1, t2, D, ldd, d_gdir, d_gxch, ldf, st,
                                    c->d_Ddf, 2, false);
          else if (r.kind == KIND_TC)
            rc = launch_quartets_tc(c, q, r.count, t1, t2, D, ldd, d_gdir, d_gxch, ldf, st, 2,
                                    r.n1, r.n2);
          else
            rc = launch_quartets_fp64(c, q, r.count, t1, t2, D, ldd, d_gdir, d_gxch, ldf, st, 2,
                                      nullptr);
          if (rc) break;
        }
      else
        rc = launch_quartets(c, c->d_quart[k], c->nquart[k], t1, t2, (const double2 *)d_dent,
                             ldd, d_gdir, d_gxch, ldf, st, 2);
      if (rc) return rc;
    }
  k_herm_complete<<<dim3(1, 256), 256, 0, st>>>((double2 *)d_gdir, c->ndim, ldf, nullptr,
                                                nullptr, 1);
  k_herm_complete<<<dim3(1, 256), 256, 0, st>>>((double2 *)d_gxch, c->ndim, ldf, nullptr,
                                                nullptr, 1);
  CK(c, cudaGetLastError());
  c->launches += 2;
  return BG_OK;
}

int bertha_gpu_clmfast(bg_ctx *c, const double *dent, int ldd, int ilev, double *gdir,
                       double *gxch, int ldf) {
  if (!c || !dent || !gdir || !gxch) return BG_ERR_ARG;
  if (c->bad) return BG_ERR_STATE;
  if (int rd = wrong_device(c)) return rd;
  if (ilev < 1 || ilev > 4 || ldd < c->ndim || ldf < c->ndim) return BG_ERR_ARG;
  if (c->hmlt == BG_HMLT_BARE) return BG_OK;
  int n = c->ndim;
  size_t bytes = sizeof(double2) * (size_t)n * n;
  if (!c->d_D) {
    CK(c, cudaMalloc(&c->d_D, bytes));
    CK(c, cudaMalloc(&c->d_GD, bytes));
    CK(c, cudaMalloc(&c->d_GX, bytes));
  }
  CK(c, cudaMemcpy2D(c->d_D, sizeof(double2) * n, dent, sizeof(double2) * ldd,
                     sizeof(double2) * n, n, cudaMemcpyHostToDevice));
  int rc = bertha_gpu_clmfast_device(c, (const double *)c->d_D, n, ilev, (double *)c->d_GD,
                                     (double *)c->d_GX, n, nullptr);
  if (rc) return rc;
  CK(c, cudaMemcpy2D(gdir, sizeof(double2) * ldf, c->d_GD, sizeof(double2) * n,
                     sizeof(double2) * n, n, cudaMemcpyDeviceToHost));
  CK(c, cudaMemcpy2D(gxch, sizeof(double2) * ldf, c->d_GX, sizeof(double2) * n,
                     sizeof(double2) * n, n, cudaMemcpyDeviceToHost));
  return BG_OK;
}

int bertha_gpu_brtfast_device(bg_ctx *c, const double *d_dent, int ldd, int ilev,
                              double *d_bxch, int ldf, void *stream) {
  if (!c) return BG_ERR_ARG;
  if (c->bad) return BG_ERR_STATE;
  if (int rd = wrong_device(c)) return rd;
  if (ilev < 1 || ilev > 4 || ldd < c->ndim || ldf < c->ndim) return BG_ERR_ARG;
  if (c->hmlt == BG_HMLT_NORL || c->hmlt == BG_HMLT_BARE) {
    c->err = "bertha_gpu_brtfast: the Breit interaction needs a four-component Hamiltonian";
    return BG_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  c->launches = 0;
  int rc = breit_prepare(c);
  if (rc) return rc;
  k_zero2d<<<1024, 256, 0, st>>>(d_bxch, c->ndim, ldf);
  CK(c, cudaGetLastError());
  c->launches++;
  // bounds for screening and, under BG_PREC_AUTO, for the bound decades
  if ((c->screen > 0.0 || c->prec == BG_PREC_AUTO) && c->bqbound.empty()) {
    rc = compute_breit_bounds(c, st);
    if (rc) return rc;
    c->bquart_ilev = -1;
  }
  if (c->bquart_ilev != ilev) {
    for (int k = 0; k < 2; ++k) {
      if (c->d_bquart[k]) cudaFree(c->d_bquart[k]);
      c->d_bquart[k] = nullptr;
      c->nbquart[k] = 0;
      std::vector<int> q = build_breit_quartets(c, k, ilev, &c->bseg[k], &c->bsegkey[k]);
      c->nbquart[k] = (long long)q.size() / 4;
      c->bruns[k].clear();
      if (!q.empty()) {
        CK(c, cudaMalloc(&c->d_bquart[k], sizeof(int) * q.size()));
        CK(c, cudaMemcpy(c->d_bquart[k], q.data(), sizeof(int) * q.size(), cudaMemcpyHostToDevice));
      }
    }
    c->bquart_ilev = ilev;
    c->btuned = false;
  }
  const double2 *D = (const double2 *)d_dent;
  bool byrun = c->prec == BG_PREC_AUTO || c->prec == BG_PREC_TC32;
  if (byrun) {
    int n = c->ndim;
    g_gaunt_dims = c->gaunt;
    if (!c->btuned && c->prec == BG_PREC_TC32) {
      for (int k = 0; k < 2; ++k) {
        c->bruns[k] = uniform_runs(c->bseg[k], c->bsegkey[k], 0, k, KIND_TC, true);
        if (regroup_list(c->d_bquart[k], c->bseg[k], c->bsegkey[k], c->bruns[k], 0, k, true, st))
          return cuda_fail(c, cudaGetLastError(), "list regrouping");
      }
      c->btuned = true;
    }
    if (!c->btuned) {
      // per class and bound decade: FP64 or tensor cores within the error
      // budget, timed and checked into a scratch output
      double *bx = nullptr, *d_e = nullptr;
      CK(c, cudaMalloc(&bx, sizeof(double2) * (size_t)n * n));
      CK(c, cudaMalloc(&d_e, 2 * sizeof(double)));
      auto zero = [&]() {
        return cudaMemsetAsync(bx, 0, sizeof(double2) * (size_t)n * n, st) == cudaSuccess ? 0 : -1;
      };
      auto energy = [&](double &ej, double &ek) {
        if (cudaMemsetAsync(d_e, 0, 2 * sizeof(double), st) != cudaSuccess) return -1;
        k_edot<<<256, 256, 0, st>>>(D, ldd, (const double2 *)bx, n, n, nullptr, nullptr, 1, d_e);
        double h[2];
        if (cudaMemcpyAsync(h, d_e, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
          return -1;
        ej = 0.0;
        ek = h[0];
        return 0;
      };
      c->btune_rec.clear();
      for (int k = 0; k < 2 && !rc; ++k) {
        const int *q = c->d_bquart[k];
        // the budget is shared by the two component classes
        rc = tune_runs(q, c->bseg[k], c->bsegkey[k], 0, k, st, 0.5 * c->err_budget,
                       [&](int kind, const int *qq, long long m, int n1, int n2) {
          if (kind == KIND_TC)
            return launch_breit_tc(c, qq, m, 0, k, D, ldd, bx, n, st, 2, n1, n2);
          return launch_breit(c, qq, m, 0, k, D, ldd, bx, n, st, 2);
        }, zero, energy, c->bruns[k], true, &c->btune_rec);
      }
      cudaFree(bx);
      cudaFree(d_e);
      if (rc) return rc > 0 ? rc : cuda_fail(c, cudaGetLastError(), "Breit autotuning");
      for (int k = 0; k < 2; ++k)
        if (regroup_list(c->d_bquart[k], c->bseg[k], c->bsegkey[k], c->bruns[k], 0, k, true, st))
          return cuda_fail(c, cudaGetLastError(), "list regrouping");
      c->btuned = true;
    }
  }
  for (int k = 0; k < 2; ++k) {
    if (byrun) {
      for (const Run &r : c->bruns[k]) {
        const int *q = c->d_bquart[k] + 4 * r.start;
        rc = r.kind == KIND_TC
                 ? launch_breit_tc(c, q, r.count, 0, k, D, ldd, d_bxch, ldf, st, 2, r.n1, r.n2)
                 : launch_breit(c, q, r.count, 0, k, D, ldd, d_bxch, ldf, st, 2);
        if (rc) return rc;
      }
    } else {
      rc = launch_breit(c, c->d_bquart[k], c->nbquart[k], 0, k, D, ldd, d_bxch, ldf, st, 2);
      if (rc) return rc;
    }
  }
  int n = c->nskp;
  // LL and SS blocks: add the (dc|ba) images of the halved (LS|SL) list
  k_herm_complete<<<dim3(1, 256), 256, 0, st>>>((double2 *)d_bxch, n, ldf, nullptr, nullptr, 1);
  k_herm_complete<<<dim3(1, 256), 256, 0, st>>>((double2 *)d_bxch + n + (size_t)ldf * n, n, ldf,
                                                nullptr, nullptr, 1);
  CK(c, cudaGetLastError());
  c->launches += 2;
  k_conj_block<<<1024, 256, 0, st>>>((double2 *)d_bxch, n, ldf);
  CK(c, cudaGetLastError());
  c->launches++;
  return BG_OK;
}

int bertha_gpu_brtfast(bg_ctx *c, const double *dent, int ldd, int ilev, double *bxch,
                       int ldf) {
  if (!c || !dent || !bxch) return BG_ERR_ARG;
  if (c->bad) return BG_ERR_STATE;
  if (int rd = wrong_device(c)) return rd;
  if (ilev < 1 || ilev > 4 || ldd < c->ndim || ldf < c->ndim) return BG_ERR_ARG;
  if (c->hmlt == BG_HMLT_NORL || c->hmlt == BG_HMLT_BARE) {
    c->err = "bertha_gpu_brtfast: the Breit interaction needs a four-component Hamiltonian";
    return BG_ERR_ARG;
  }
  int n = c->ndim;
  size_t bytes = sizeof(double2) * (size_t)n * n;
  if (!c->d_D) {
    CK(c, cudaMalloc(&c->d_D, bytes));
    CK(c, cudaMalloc(&c->d_GD, bytes));
    CK(c, cudaMalloc(&c->d_GX, bytes));
  }
  if (!c->d_BX) CK(c, cudaMalloc(&c->d_BX, bytes));
  CK(c, cudaMemcpy2D(c->d_D, sizeof(double2) * n, dent, sizeof(double2) * ldd,
                     sizeof(double2) * n, n, cudaMemcpyHostToDevice));
  int rc = bertha_gpu_brtfast_device(c, (const double *)c->d_D, n, ilev, (double *)c->d_BX, n,
                                     nullptr);
  if (rc) return rc;
  CK(c, cudaMemcpy2D(bxch, sizeof(double2) * ldf, c->d_BX, sizeof(double2) * n,
                     sizeof(double2) * n, n, cudaMemcpyDeviceToHost));
  return BG_OK;
}

int bertha_gpu_oneel_device(bg_ctx *c, const double *znuc, const double *xi, double *d_ovlp,
                             double *d_hnuc, double *d_hkin, int ldf, void *stream) {
  if (!c || !znuc || !xi || !d_ovlp || !d_hnuc || !d_hkin) return BG_ERR_ARG;
  if (c->bad) return BG_ERR_STATE;
  if (int rd = wrong_device(c)) return rd;
  if (ldf < c->ndim) return BG_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  std::vector<double> nuc((size_t)c->ncnt * 5);
  for (int i = 0; i < c->ncnt; ++i) {
    if (!(xi[i] >= 0.0)) return BG_ERR_ARG;
    for (int x = 0; x < 3; ++x) nuc[5 * i + x] = c->cxyz[3 * i + x];
    nuc[5 * i + 3] = znuc[i];
    nuc[5 * i + 4] = xi[i];
  }
  double *d_nuc = nullptr;
  CK(c, cudaMalloc(&d_nuc, sizeof(double) * nuc.size()));
  CK(c, cudaMemcpyAsync(d_nuc, nuc.data(), sizeof(double) * nuc.size(), cudaMemcpyHostToDevice, st));
  c->launches = 0;
  k_zero2d<<<1024, 256, 0, st>>>(d_ovlp, c->ndim, ldf);
  k_zero2d<<<1024, 256, 0, st>>>(d_hnuc, c->ndim, ldf);
  k_zero2d<<<1024, 256, 0, st>>>(d_hkin, c->ndim, ldf);
  k_oneel<<<(unsigned)((long long)c->ns * c->ns), 64, 0, st>>>(
      c->d_sh, c->ns, c->d_pe, c->d_E, d_nuc, c->ncnt, c->nskp, c->hmlt == BG_HMLT_NORL,
      (double2 *)d_ovlp, (double2 *)d_hnuc, (double2 *)d_hkin, ldf);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d_nuc);
  if (e != cudaSuccess) return cuda_fail(c, e, "k_oneel");
  c->launches += 4;
  return BG_OK;
}

int bertha_gpu_oneel(bg_ctx *c, const double *znuc, const double *xi, double *ovlp,
                     double *hnuc, double *hkin, int ldf) {
  if (!c || !ovlp || !hnuc || !hkin) return BG_ERR_ARG;
  if (c->bad) return BG_ERR_STATE;
  if (int rd = wrong_device(c)) return rd;
  if (ldf < c->ndim) return BG_ERR_ARG;
  int n = c->ndim;
  size_t bytes = sizeof(double2) * (size_t)n * n;
  double *d[3] = {nullptr, nullptr, nullptr};
  for (int k = 0; k < 3; ++k) {
    cudaError_t e = cudaMalloc(&d[k], bytes);
    if (e != cudaSuccess) {
      for (int j = 0; j < k; ++j) cudaFree(d[j]);
      return cuda_fail(c, e, "cudaMalloc");
    }
  }
  int rc = bertha_gpu_oneel_device(c, znuc, xi, d[0], d[1], d[2], n, nullptr);
  double *h[3] = {ovlp, hnuc, hkin};
  for (int k = 0; k < 3 && rc == BG_OK; ++k) {
    cudaError_t e = cudaMemcpy2D(h[k], sizeof(double2) * ldf, d[k], sizeof(double2) * n,
                                 sizeof(double2) * n, n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = cuda_fail(c, e, "cudaMemcpy2D");
  }
  for (int k = 0; k < 3; ++k) cudaFree(d[k]);
  return rc;
}

void bertha_gpu_free(bg_ctx *c) {
  if (!c) return;
  cudaFree(c->d_sh);
  cudaFree(c->d_pe);
  cudaFree(c->d_E);
  for (int k = 0; k < 4; ++k) cudaFree(c->d_quart[k]);
  cudaFree(c->d_Edf);
  cudaFree(c->d_Ef);
  cudaFree(c->d_Ddf);
  cudaFree(c->d_qp);
  cudaFree(c->d_D);
  cudaFree(c->d_GD);
  cudaFree(c->d_GX);
  cudaFree(c->d_EB);
  cudaFree(c->d_EBf);
  cudaFree(c->d_offq);
  for (int k = 0; k < 2; ++k) {
    if (c->h_chunk[k]) cudaFreeHost(c->h_chunk[k]);
    cudaFree(c->d_chunk[k]);
    if (c->chunk_ev[k]) cudaEventDestroy(c->chunk_ev[k]);
  }
  cudaFree(c->d_Ecv);
  cudaFree(c->d_Eci);
  cudaFree(c->d_EBcv);
  cudaFree(c->d_EBci);
  for (int k = 0; k < 2; ++k) cudaFree(c->d_bquart[k]);
  cudaFree(c->d_BX);
  delete c;
}

int bertha_gpu_batch_create(bg_batch **out, int n, bg_ctx *const *ctxs,
                            const long long *moff, const int *ld) {
  if (!out) return BG_ERR_ARG;
  *out = nullptr;
  if (n < 1 || !ctxs) { g_init_err = "invalid argument"; return BG_ERR_ARG; }
  for (int i = 0; i < n; ++i) {
    if (!ctxs[i]) { g_init_err = "null context"; return BG_ERR_ARG; }
    if (ctxs[i]->bad) { g_init_err = "context failed earlier"; return BG_ERR_STATE; }
    const bg_ctx *c = ctxs[i], *c0 = ctxs[0];
    if (c->dev != c0->dev || c->dev != current_device()) {
      g_init_err = "batched instances must live on the current device";
      return BG_ERR_STATE;
    }
    if (c->hmlt != c0->hmlt || c->isym != c0->isym || c->racah1 != c0->racah1) {
      g_init_err = "batched instances must share hmlt, shape and the RACAH1 flag";
      return BG_ERR_ARG;
    }
  }
  for (int i = 0; i < n; ++i) {
    bg_ctx *c = ctxs[i];
    if (c->screen > 0.0 && c->qbound.empty()) {
      int rc = compute_bounds(c, nullptr);
      if (rc) { g_init_err = c->err; return rc; }
    }
  }
  bg_batch *b = new bg_batch();
  b->dev = ctxs[0]->dev;
  b->n = n;
  b->ncomp = ctxs[0]->ncomp; b->hmlt = ctxs[0]->hmlt; b->isym = ctxs[0]->isym;
  b->racah1 = ctxs[0]->racah1; b->prec = ctxs[0]->prec; b->err_budget = ctxs[0]->err_budget;
  std::vector<long long> pbase(n), ebase(n);
  long long nst = 0, npt = 0, net = 0, packed = 0;
  std::vector<Shell> sh;
  for (int i = 0; i < n; ++i) {
    const bg_ctx *c = ctxs[i];
    b->sbase.push_back((int)nst);
    pbase[i] = npt;
    ebase[i] = net;
    Inst I;
    I.off = moff ? moff[i] : packed;
    I.ld = ld ? ld[i] : c->ndim;
    I.nskp = c->nskp;
    if (I.off < 0 || I.ld < c->ndim) {
      g_init_err = "invalid placement of instance " + std::to_string(i);
      bertha_gpu_batch_free(b);
      return BG_ERR_ARG;
    }
    b->inst.push_back(I);
    b->ndim.push_back(c->ndim);
    if (c->ndim > 0)
      b->span = std::max(b->span, I.off + (long long)I.ld * (c->ndim - 1) + c->ndim);
    packed += (long long)c->ndim * c->ndim;
    for (int a = 0; a < c->ns; ++a) {
      Shell s2 = c->shells[a];
      s2.inst = i;
      s2.prow = (int)(npt + (long long)a * c->ns - nst);
      sh.push_back(s2);
    }
    nst += c->ns;
    npt += (long long)c->ns * c->ns;
    net += c->nE;
    if (npt > 0x7fffffffLL) {
      g_init_err = "batch pair table beyond 2^31 entries";
      bertha_gpu_batch_free(b);
      return BG_ERR_CAPACITY;
    }
    bg_ctx *h = new bg_ctx();
    h->ns = c->ns; h->ncomp = c->ncomp; h->racah1 = c->racah1;
    h->shells = c->shells; h->qbound = c->qbound; h->screen = c->screen;
    b->shadow.push_back(h);
  }
  cudaError_t e = cudaSuccess;
  auto fail = [&](const char *what) {
    g_init_err = std::string(what) + ": " + cudaGetErrorString(e);
    bertha_gpu_batch_free(b);
    return BG_ERR_CUDA;
  };
  if ((e = cudaMalloc(&b->d_sh, sizeof(Shell) * std::max<long long>(nst, 1))) ||
      (e = cudaMalloc(&b->d_pe, sizeof(PairE) * std::max<long long>(npt, 1))) ||
      (e = cudaMalloc(&b->d_E, sizeof(double2) * std::max<long long>(net, 1))) ||
      (e = cudaMalloc(&b->d_Ecv, sizeof(double2) * std::max<long long>(net, 1))) ||
      (e = cudaMalloc(&b->d_Eci, std::max<long long>(net, 1))) ||
      (e = cudaMalloc(&b->d_Edf, sizeof(float4) * std::max<long long>(net, 1))) ||
      (e = cudaMalloc(&b->d_Ef, sizeof(float2) * std::max<long long>(net, 1))) ||
      (e = cudaMalloc(&b->d_inst, sizeof(Inst) * n)) ||
      (e = cudaMalloc(&b->d_ndim, sizeof(int) * n)))
    return fail("cudaMalloc");
  if ((e = cudaMemcpy(b->d_sh, sh.data(), sizeof(Shell) * nst, cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(b->d_inst, b->inst.data(), sizeof(Inst) * n, cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(b->d_ndim, b->ndim.data(), sizeof(int) * n, cudaMemcpyHostToDevice)))
    return fail("cudaMemcpy");
  for (int i = 0; i < n; ++i) {
    const bg_ctx *c = ctxs[i];
    long long np = (long long)c->ns * c->ns, ne = c->nE;
    std::vector<PairE> pe(np);
    if ((e = cudaMemcpy(pe.data(), c->d_pe, sizeof(PairE) * np, cudaMemcpyDeviceToHost)))
      return fail("cudaMemcpy");
    for (PairE &p : pe)
      for (int t = 0; t < 2; ++t)
        if (p.off[t] >= 0) p.off[t] += ebase[i];
    if ((e = cudaMemcpy(b->d_pe + pbase[i], pe.data(), sizeof(PairE) * np,
                        cudaMemcpyHostToDevice)))
      return fail("cudaMemcpy");
    if (ne > 0 &&
        ((e = cudaMemcpy(b->d_E + ebase[i], c->d_E, sizeof(double2) * ne, cudaMemcpyDeviceToDevice)) ||
         (e = cudaMemcpy(b->d_Ecv + ebase[i], c->d_Ecv, sizeof(double2) * ne, cudaMemcpyDeviceToDevice)) ||
         (e = cudaMemcpy(b->d_Eci + ebase[i], c->d_Eci, ne, cudaMemcpyDeviceToDevice)) ||
         (e = cudaMemcpy(b->d_Edf + ebase[i], c->d_Edf, sizeof(float4) * ne, cudaMemcpyDeviceToDevice)) ||
         (e = cudaMemcpy(b->d_Ef + ebase[i], c->d_Ef, sizeof(float2) * ne, cudaMemcpyDeviceToDevice))))
      return fail("cudaMemcpy");
  }
  *out = b;
  return BG_OK;
}

int bertha_gpu_batch_set_precision(bg_batch *b, int prec) {
  if (!b) return BG_ERR_ARG;
  if (prec != BG_PREC_FP64 && prec != BG_PREC_DF32 && prec != BG_PREC_AUTO &&
      prec != BG_PREC_TC32)
    return BG_ERR_ARG;
  if (prec != b->prec) b->tuned = false;
  b->prec = prec;
  return BG_OK;
}

int bertha_gpu_batch_clmfast_device(bg_batch *b, const double *d_dent, int ilev, double *d_gdir,
                                    double *d_gxch, void *stream) {
  if (!b) return BG_ERR_ARG;
  if (b->bad) return BG_ERR_STATE;
  if (current_device() != b->dev) {
    b->err = "batch was made on device " + std::to_string(b->dev) + ", another device is current";
    return BG_ERR_STATE;
  }
  if (ilev < 1 || ilev > 4 || !d_dent || !d_gdir || !d_gxch) return BG_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  b->launches = 0;
  if (b->hmlt == BG_HMLT_BARE) return BG_OK;
  unsigned gx = (unsigned)std::min(b->n, 1024);
  k_zero_inst<<<dim3(gx, 16), 256, 0, st>>>(d_gdir, b->d_inst, b->d_ndim, b->n);
  k_zero_inst<<<dim3(gx, 16), 256, 0, st>>>(d_gxch, b->d_inst, b->d_ndim, b->n);
  BK(b, cudaGetLastError());
  b->launches += 2;
  if (b->quart_ilev != ilev) {
    int rc = batch_lists(b, ilev);
    if (rc) return rc;
  }
  if (b->prec == BG_PREC_DF32 || b->prec == BG_PREC_AUTO) {
    if (!b->d_Ddf) BK(b, cudaMalloc(&b->d_Ddf, sizeof(float4) * std::max<long long>(b->span, 1)));
    k_dconv1<<<1024, 256, 0, st>>>((const double2 *)d_dent, b->span, b->d_Ddf);
    BK(b, cudaGetLastError());
    b->launches++;
  }
  const double2 *D = (const double2 *)d_dent;
  if (b->prec == BG_PREC_AUTO && !b->tuned) {
    // kernel choice per angular class, timed and checked into scratch outputs
    double *gd = nullptr, *gx = nullptr, *d_e = nullptr;
    size_t bytes = sizeof(double2) * std::max<long long>(b->span, 1);
    BK(b, cudaMalloc(&gd, bytes));
    BK(b, cudaMalloc(&gx, bytes));
    BK(b, cudaMalloc(&d_e, 2 * sizeof(double)));
    auto zero = [&]() {
      if (cudaMemsetAsync(gd, 0, bytes, st) != cudaSuccess ||
          cudaMemsetAsync(gx, 0, bytes, st) != cudaSuccess)
        return -1;
      return 0;
    };
    auto energy = [&](double &ej, double &ek) {
      if (cudaMemsetAsync(d_e, 0, 2 * sizeof(double), st) != cudaSuccess) return -1;
      k_edot<<<256, 256, 0, st>>>(D, 0, (const double2 *)gd, 0, 0, b->d_inst, b->d_ndim, b->n,
                                  d_e);
      k_edot<<<256, 256, 0, st>>>(D, 0, (const double2 *)gx, 0, 0, b->d_inst, b->d_ndim, b->n,
                                  d_e + 1);
      double h[2];
      if (cudaMemcpyAsync(h, d_e, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess)
        return -1;
      ej = h[0];
      ek = h[1];
      return 0;
    };
    int rc = 0;
    for (int t1 = 0; t1 < b->ncomp && !rc; ++t1)
      for (int t2 = 0; t2 < b->ncomp && !rc; ++t2) {
        int k = 2 * t1 + t2;
        double budget = b->err_budget / (b->ncomp * b->ncomp);
        rc = tune_runs(b->d_quart[k], b->seg[k], b->segkey[k], t1, t2, st, budget,
                       [&](int kind, const int *qq, long long m, int n1, int n2) {
          return batch_launch(b, t1, t2, kind, (const int4 *)qq, m, D, gd, gx, st, n1, n2);
        }, zero, energy, b->runs[k]);
      }
    cudaFree(gd);
    cudaFree(gx);
    cudaFree(d_e);
    if (rc) return rc > 0 ? rc : batch_fail(b, cudaGetLastError(), "autotuning");
    for (int t1 = 0; t1 < b->ncomp; ++t1)
      for (int t2 = 0; t2 < b->ncomp; ++t2) {
        int k = 2 * t1 + t2;
        if (regroup_list(b->d_quart[k], b->seg[k], b->segkey[k], b->runs[k], t1, t2, false, st))
          return batch_fail(b, cudaGetLastError(), "list regrouping");
      }
    b->tuned = true;
  }
  if (b->prec == BG_PREC_TC32 && !b->tuned) {
    for (int t1 = 0; t1 < b->ncomp; ++t1)
      for (int t2 = 0; t2 < b->ncomp; ++t2) {
        int k = 2 * t1 + t2;
        b->runs[k] = uniform_runs(b->seg[k], b->segkey[k], t1, t2, KIND_TC);
        if (regroup_list(b->d_quart[k], b->seg[k], b->segkey[k], b->runs[k], t1, t2, false, st))
          return batch_fail(b, cudaGetLastError(), "list regrouping");
      }
    b->tuned = true;
  }
  for (int t1 = b->ncomp - 1; t1 >= 0; --t1)
    for (int t2 = b->ncomp - 1; t2 >= 0; --t2) {
      int k = 2 * t1 + t2, rc = 0;
      if (b->prec == BG_PREC_AUTO || b->prec == BG_PREC_TC32)
        for (const Run &r : b->runs[k]) {
          rc = batch_launch(b, t1, t2, r.kind, (const int4 *)b->d_quart[k] + r.start, r.count, D,
                            d_gdir, d_gxch, st, r.n1, r.n2);
          if (rc) break;
        }
      else
        rc = batch_launch(b, t1, t2, b->prec == BG_PREC_DF32 ? KIND_DF32 : KIND_FP64,
                          (const int4 *)b->d_quart[k], b->nquart[k], D, d_gdir, d_gxch, st);
      if (rc) return rc;
    }
  k_herm_complete<<<dim3(gx, 16), 256, 0, st>>>((double2 *)d_gdir, 0, 0, b->d_inst, b->d_ndim,
                                                b->n);
  k_herm_complete<<<dim3(gx, 16), 256, 0, st>>>((double2 *)d_gxch, 0, 0, b->d_inst, b->d_ndim,
                                                b->n);
  BK(b, cudaGetLastError());
  b->launches += 2;
  return BG_OK;
}

long long bertha_gpu_batch_quartets(const bg_batch *b) {
  if (!b) return 0;
  return b->nquart[0] + b->nquart[1] + b->nquart[2] + b->nquart[3];
}

long long bertha_gpu_batch_launches(const bg_batch *b) { return b ? b->launches : 0; }

const char *bertha_gpu_batch_last_error(const bg_batch *b) {
  return b ? b->err.c_str() : g_init_err.c_str();
}

void bertha_gpu_batch_free(bg_batch *b) {
  if (!b) return;
  for (bg_ctx *h : b->shadow) delete h;
  cudaFree(b->d_sh);
  cudaFree(b->d_pe);
  cudaFree(b->d_E);
  cudaFree(b->d_Ecv);
  cudaFree(b->d_Eci);
  cudaFree(b->d_Edf);
  cudaFree(b->d_Ef);
  cudaFree(b->d_Ddf);
  cudaFree(b->d_qp);
  cudaFree(b->d_inst);
  cudaFree(b->d_ndim);
  for (int k = 0; k < 4; ++k) cudaFree(b->d_quart[k]);
  delete b;
}

}  // extern "C"

// Tensor-core quartet kernel: the two Hermite contractions of ERIFAST
// (bertha-scf.f:12676-12799 first, :12802-13126 second) as GEMMs on the
// 5th-generation tensor cores (tcgen05.mma kind::tf32, accumulators in
// tensor memory), each product in three TF32 passes hi*hi + hi*lo + lo*hi
// (3xTF32, about 22 significant bits per operand, FP32 accumulation).
// Boys values and the R recursion stay FP64 (as in k_quartet_df), the
// per-quartet J/K sums are FP32 and every J/K element is accumulated in FP64
// in global memory.  Included inside the anonymous namespace of
// bertha_gpu.cu.
//
// One CTA (256 threads, or 512 for classes that take a whole SM's tensor
// memory) per shell quartet (grid-stride).  With the left pair
// (labels L, Hermite terms s) and the right pair (labels R, terms q):
//   GEMM 1  D1[row][q]   = sum_s  E_L[row][s] * R[s+q]        rows (L, set, re/im)
//   GEMM 2  D2[row][col] = sum_q  G[row][q] * E_R[col][q]     cols (R, set, re/im)
// with G = D1 times (-1)^|q| and the exponent balancing of the split path.
// M = 128 rows per tile (32 left labels), K in chunks of 32, B operands K-major.
// D2 holds, per label pair, the 16 real products that ERIFAST's second
// contraction forms (:12809-13119); the 16 m-sign combinations and the
// CLMMTG/CLMMTZ digestion (batch types 1 and 5) follow in FP32.

namespace tcq {

constexpr int KC = 32;          // K elements per staged chunk (4 MMAs of K = 8)
constexpr int MROWS = 128;      // rows per M tile
constexpr int MLAB = MROWS / 4; // left labels per M tile
constexpr int N1MAX = 192;      // roundup(165, 32): R columns of the right pair
constexpr int N2MAX = 208;      // roundup(4 * 49, 16): E columns of the right pair
constexpr int PSTR = 65;        // row stride (floats) of the D2 slab in shared memory
constexpr int SLAB = 64;        // D2 columns per epilogue slab (16 right labels)
constexpr long long WAIT_LIMIT = 1LL << 24;  // mbarrier polls before giving up

__device__ int g_tc_status;  // nonzero: a tensor-core wait timed out or a class did not fit

__device__ __forceinline__ uint32_t saddr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor of a K-major operand without swizzling:
// core matrices of 8 rows x 16 bytes, stored contiguously (128 B); the two
// core matrices of one MMA's K = 8 extent 128 B apart (leading byte offset),
// 8-row groups 1024 B apart (stride byte offset: a 32-element chunk holds 8
// core matrices per row group); bits 46-48 carry the fixed value 0b001.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
  return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)(128 >> 4) << 16) |
         ((uint64_t)(1024 >> 4) << 32) | ((uint64_t)1 << 46);
}

// Instruction descriptor, kind::tf32: FP32 accumulator, TF32 A and B,
// both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__device__ __forceinline__ uint32_t idesc(int m, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}

// Float offset of element (row, k) of a staged K chunk: [row/8][k/4][row%8][k%4].
__device__ __forceinline__ int kmaj(int row, int k) {
  return (((row >> 3) * (KC / 4) + (k >> 2)) * 8 + (row & 7)) * 4 + (k & 3);
}

// TF32 value of x rounded to nearest (ties away from zero).
__device__ __forceinline__ float tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// x = hi + lo, both TF32 and rounded to nearest, ~22 significant bits in
// all: rounding (not truncation) keeps the dropped parts of unbiased sign,
// so the products' errors average out in the J/K sums instead of drifting.
__device__ __forceinline__ void tsplit(float x, float &h, float &l) {
  h = tf32(x);
  l = tf32(x - h);
}

// Hermite index tables in shared memory: t | u << 8 | v << 16 | lambda << 24
// (a lane-divergent __constant__ read would be serialised).
__device__ __forceinline__ int tuvL(uint32_t w) { return (int)(w >> 24); }
__device__ __forceinline__ int hsum(uint32_t a, uint32_t b) {
  int t = (int)(a & 255) + (int)(b & 255), u = (int)((a >> 8) & 255) + (int)((b >> 8) & 255);
  int v = (int)((a >> 16) & 255) + (int)((b >> 16) & 255);
  return hidx(t, u, v);
}

__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id,
                                    uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred pa;\n\t"
      "setp.ne.b32 pa, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, pa;\n\t}"
      :: "r"(d), "l"(a), "l"(b), "r"(id), "r"(acc));
}

__device__ __forceinline__ void commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
               :: "r"(saddr(bar)) : "memory");
}

// Waits for completion of the phase with the given parity; false after
// WAIT_LIMIT polls.
__device__ __forceinline__ bool wait(uint64_t *bar, uint32_t parity) {
  uint32_t done = 0;
  for (long long it = 0; it < WAIT_LIMIT && !done; ++it)
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done) : "r"(saddr(bar)), "r"(parity) : "memory");
  return done != 0;
}

__device__ __forceinline__ void fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 8 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tld8(uint32_t ta, float *v) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7])
      : "r"(ta));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 8; ++j) v[j] = __uint_as_float(r[j]);
}

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tld16(uint32_t ta, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(ta));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}


__host__ __device__ inline int rup(int x, int m) { return (x + m - 1) / m * m; }

// Tensor-core cost (MMA columns x K, per 128-row tile) of an orientation:
// left pair nlL labels / nL terms, right pair nlR / nR.
__host__ __device__ inline long long tc_cost(int nlL, int nL, int nlR, int nR) {
  long long tiles = (4 * nlL + MROWS - 1) / MROWS;
  int n1 = rup(nR, KC), n2 = rup(4 * nlR, 16);
  return tiles * ((long long)rup(nL, KC) * n1 + (long long)n1 * n2) + 64LL * nlL * nlR;
}

// TMEM columns (D1, D2) a class needs in the orientation the kernel takes.
__host__ __device__ inline void tc_dims(int la, int lb, int lc, int ld, int t1, int t2, int &n1,
                                        int &n2, bool &swp) {
  int nab = ntuv(la + lb + 2 * t1), ncd = ntuv(lc + ld + 2 * t2);
  int nlab = (2 * la + 1) * (2 * lb + 1), nlcd = (2 * lc + 1) * (2 * ld + 1);
  swp = tc_cost(nlcd, ncd, nlab, nab) < tc_cost(nlab, nab, nlcd, ncd);
  int nR = swp ? nab : ncd, nlR = swp ? nlab : nlcd;
  n1 = rup(nR, KC);
  n2 = rup(4 * nlR, 16);
}

// Tensor-core cost of a Breit orientation (as tc_cost, three components i,
// each contracting three components j, or one for the Gaunt term alone).
__host__ __device__ inline long long tcb_cost(int nlL, int nL, int nlR, int nR, int gaunt) {
  long long tiles = (4 * nlL + MROWS - 1) / MROWS;
  int n1 = rup(nR, KC), n2 = rup(4 * nlR, 16);
  int nj = gaunt ? 1 : 3;
  return tiles * 3 * ((long long)nj * rup(nL, KC) * n1 + (long long)n1 * n2) + 64LL * nlL * nlR;
}

__host__ __device__ inline void tcb_dims(int la, int lb, int lc, int ld, int gaunt, int &n1,
                                         int &n2, bool &swp) {
  int nab = ntuv(la + lb + 1), ncd = ntuv(lc + ld + 1);
  int nlab = (2 * la + 1) * (2 * lb + 1), nlcd = (2 * lc + 1) * (2 * ld + 1);
  swp = tcb_cost(nlcd, ncd, nlab, nab, gaunt) < tcb_cost(nlab, nab, nlcd, ncd, gaunt);
  int nR = swp ? nab : ncd, nlR = swp ? nlab : nlcd;
  n1 = rup(nR, KC);
  n2 = rup(4 * nlR, 16);
}

constexpr int NWT = ntuv(4 * BG_MAX_L + 2);  // Breit kernel-table entries (degree la+lb+lc+ld+2)
constexpr int ABYTES = 2 * MROWS * KC * 4;    // one A staging buffer (hi and lo)

// Shared-memory layout (bytes from a 128-byte aligned base):
//   nbuf A buffers (MROWS x KC, hi and lo; their padding rows stay zero, so
//   that a staging pass only writes the rows that carry data),
//   nbuf B buffers of bbytes each, whose space the FP64 R recursion (before
//   the GEMMs) and the D2 slab (after them) reuse,
//   the table the B operand is read from (R, or the Breit kernel table),
//   nblk density blocks and nblk J/K accumulators, the Boys values.
// Double buffering (nbuf = 2) lets the next K chunk be staged while the
// tensor cores work on the current one.
struct Layout {
  int abuf, bbuf, bsz, rf, dsm, acc, fb, total;
};
__host__ __device__ inline Layout layout(int bbytes, int nbuf, int rfbytes, int nblk,
                                          int accb) {
  Layout L;
  L.abuf = 0;
  L.bsz = rup(bbytes, 128);
  int breg = nbuf * L.bsz;
  breg = breg > MROWS * PSTR * 4 ? breg : MROWS * PSTR * 4;  // D2 slab
  breg = breg > 2 * NTR * 8 ? breg : 2 * NTR * 8;            // FP64 R recursion
  L.bbuf = nbuf * ABYTES;
  L.rf = rup(L.bbuf + breg, 128);
  L.dsm = L.rf + rup(rfbytes, 128);
  L.acc = L.dsm + nblk * MAXSP * MAXSP * 8;
  L.fb = L.acc + nblk * MAXSP * MAXSP * accb;  // accb: 8 (FP32) or 16 (FP64) per element
  L.total = L.fb + (MAXLAM + 4) * 8 + 128;  // + alignment slack
  return L;
}

// B-buffer bytes of the Coulomb kernel (one operand of up to max(n1, n2)
// rows) and of the Breit kernel (three GEMM-1 operands of n1 rows when the
// three Cartesian components run together, else one).
__host__ __device__ inline int bbytes_c(int n1, int n2) {
  return 2 * (n1 > n2 ? n1 : n2) * KC * 4;
}
__host__ __device__ inline int bbytes_b(int n1, int n2, int tri) {
  int b1 = (tri ? 3 : 1) * 2 * n1 * KC * 4, b2 = 2 * n2 * KC * 4;
  return b1 > b2 ? b1 : b2;
}
__host__ __device__ inline Layout layout_c(int n1, int n2, int nbuf, bool f64acc) {
  return layout(bbytes_c(n1, n2), nbuf, NTR * 4, 4, f64acc ? 16 : 8);
}
__host__ __device__ inline Layout layout_b(int n1, int n2, int nbuf, int tri) {
  return layout(bbytes_b(n1, n2, tri), nbuf, NWT * 6 * 4, 2, 16);
}

// MMA completion tracking of up to two staging buffers: one mbarrier per
// buffer, its phase parity, and whether a commit on it is outstanding.
struct Pipe {
  uint64_t *bar;
  uint32_t ph[2];
  bool pend[2];
};

// Waits for the outstanding commit on buffer b (if any); false on timeout.
__device__ __forceinline__ bool pipe_wait(Pipe &p, int b) {
  if (!p.pend[b]) return true;
  bool ok = wait(&p.bar[b], p.ph[b]);
  p.ph[b] ^= 1;
  p.pend[b] = false;
  return ok;
}

struct Args {
  const Shell *sh;
  const PairE *pe;
  const float2 *E;   // FP32 E copy (re, im), scaled like the double-float copy
  const double2 *D;  // density as the caller holds it, leading dimension ldd (batched: Inst placement)
  double *GD, *GX;
  int ldd, ldf, nskp, isym, racah1;
  int sym;           // as QArgsDF
  const Inst *inst;
  const double *qp;  // per-quartet records of k_qprep, one per list entry
  int tmem_cols, n1max, n2max, nbuf;
};

struct ArgsB {
  const Shell *sh;
  const PairE *pe;        // kexp of each ordered pair (row prow of the first shell)
  const long long *offq;  // sigma-coupled E offsets [pair][LS/SL]
  const float2 *E;        // their FP32 copy, scaled by 2^(kexp lambda)
  const double2 *D;       // density as the caller holds it, leading dimension ldd
  double *BX;
  int ns, ldd, ldf, nskp, isym, racah1, gaunt;
  int dual;               // as BArgs
  const double *qp;       // per-quartet records of k_qprep, one per list entry
  int tmem_cols, n1max, n2max, nbuf;
  int tri;                // the three Cartesian components' D1 side by side in TMEM
};

// The 16 m-sign combinations of (left|right) from the four complex products
// s_p = u*x and their conjugate-side forms sc_p = u*conj(x) (sv = s1, s1c,
// ..., s4, s4c) with the left pair phase sl and the product phase slr
// (ERIFAST :12861-12864, :13013-13016: the time-reversal relations), index
// 8a+4b+2c+d of (left|right).
__device__ __forceinline__ void combos16(const float2 (&sv)[8], float sl, float slr,
                                         float2 (&r)[16]) {
  r[0] = sv[0];
  r[12] = make_float2(sv[1].x * sl, sv[1].y * sl);
  r[15] = make_float2(r[0].x * slr, -r[0].y * slr);
  r[3] = make_float2(r[12].x * slr, -r[12].y * slr);
  r[2] = sv[2];
  r[14] = make_float2(sv[3].x * sl, sv[3].y * sl);
  r[13] = make_float2(-r[2].x * slr, r[2].y * slr);
  r[1] = make_float2(-r[14].x * slr, r[14].y * slr);
  r[8] = sv[4];
  r[4] = make_float2(-sv[5].x * sl, -sv[5].y * sl);
  r[7] = make_float2(-r[8].x * slr, r[8].y * slr);
  r[11] = make_float2(-r[4].x * slr, r[4].y * slr);
  r[10] = sv[6];
  r[6] = make_float2(-sv[7].x * sl, -sv[7].y * sl);
  r[5] = make_float2(r[10].x * slr, -r[10].y * slr);
  r[9] = make_float2(r[6].x * slr, -r[6].y * slr);
}

// The 8 complex products of a label pair from the D2 slab: rows (left label,
// set, re/im), columns (right label, set, re/im); pp = 2 setL + setR,
// s_p = u*x = (a-b, c+d), sc_p = u*conj(x) = (a+b, d-c) with a = re.re,
// b = im.im, c = G.im E.re, d = G.re E.im.
__device__ __forceinline__ void products8(const float *pr0, float2 (&sv)[8]) {
#pragma unroll
  for (int sL = 0; sL < 2; ++sL)
#pragma unroll
    for (int sR = 0; sR < 2; ++sR) {
      const float *p = pr0 + (sL * 2) * PSTR + sR * 2;
      float a = p[0], d = p[1], c = p[PSTR], b = p[PSTR + 1];
      int pp = sL * 2 + sR;
      sv[2 * pp] = make_float2(a - b, c + d);
      sv[2 * pp + 1] = make_float2(a + b, d - c);
    }
}

__device__ __forceinline__ void cmac(float2 &acc, float2 u, float2 d) {
  acc.x = fmaf(u.x, d.x, fmaf(-u.y, d.y, acc.x));
  acc.y = fmaf(u.x, d.y, fmaf(u.y, d.x, acc.y));
}

// A work item's FP32 contribution into a shared FP64 accumulator: the
// accumulation order of the items is not fixed, and in FP64 its rounding
// stays at the level of the global FP64 sums (FP32 accumulators would make
// a build's result vary by ~1e-7 between identical calls, enough to keep
// an SCF from converging to 1e-9 Eh).
__device__ __forceinline__ void sadd(double2 *p, float2 v) {
  atomicAdd(&p->x, (double)v.x);
  atomicAdd(&p->y, (double)v.y);
}
// The same into an FP32 accumulator (one-shot explicit-list digestion).
__device__ __forceinline__ void sadd(float2 *p, float2 v) {
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}

// ---- staging of one K chunk into the canonical K-major layout ----
//
// A staged operand is written in 16-byte pieces (4 consecutive K terms of one
// row), piece p at float offset 4p, so that a warp stores four whole
// 8-row x 4-term core matrices (512 contiguous bytes) and the shared-memory
// banks take the stores without conflicts.  Piece p holds row prow(p) and
// terms pk(p) .. pk(p)+3; the rows [8g, 8g+8) are the pieces [64g, 64g+64).
__device__ __forceinline__ int prow(int p) { return ((p >> 6) << 3) | (p & 7); }
__device__ __forceinline__ int pk(int p) { return ((p >> 3) & 7) << 2; }
__device__ __forceinline__ int piece(int row, int k0) {
  return ((row >> 3) << 6) | ((k0 >> 2) << 3) | (row & 7);
}

// hi and lo TF32 parts of four values into piece p of H and L.
__device__ __forceinline__ void put4(float *H, float *L, int p, const float *v) {
  float4 h, l;
  tsplit(v[0], h.x, l.x);
  tsplit(v[1], h.y, l.y);
  tsplit(v[2], h.z, l.z);
  tsplit(v[3], h.w, l.w);
  reinterpret_cast<float4 *>(H)[p] = h;
  reinterpret_cast<float4 *>(L)[p] = l;
}

// Zeroes rows [r0, r1) of a staged chunk.
template <int NT>
__device__ __forceinline__ void clear_rows(float *H, float *L, int r0, int r1, int tid) {
  const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int p = ((r0 >> 3) << 6) + tid; p < ((r1 + 7) >> 3) << 6; p += NT) {
    int row = prow(p);
    if (row >= r0 && row < r1) {
      reinterpret_cast<float4 *>(H)[p] = z;
      reinterpret_cast<float4 *>(L)[p] = z;
    }
  }
}

// A rows from E-coefficients: row (label, set, re/im) = 4 label + 2 set + ri
// for ntl labels; src is label 0 set 0 term 0, rows of (label, set) rstride
// apart; each term s scaled by sc[lambda_s] (the exponent balancing's
// power of two).  Rows from 4 ntl up to the buffer's previous row count are
// cleared (the rest are zero already).
template <int NT>
__device__ __forceinline__ void stage_e_rows(float *Ah, float *Al, const float2 *src,
                                             long long rstride, int ntl, int kc, int nK,
                                             const float *sc, const uint32_t *stuv, int &arows,
                                             int tid) {
  const int rows = 4 * ntl, r8 = (rows + 7) & ~7;
  const float *sf = reinterpret_cast<const float *>(src);
  for (int p = tid; p < r8 * (KC / 4); p += NT) {
    int row = prow(p), s0 = kc + pk(p);
    float v[4] = {0.f, 0.f, 0.f, 0.f};
    if (row < rows) {
      const float *e = sf + 2 * ((long long)(row >> 1) * rstride + s0) + (row & 1);
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (s0 + j < nK) v[j] = __ldg(e + 2 * j) * sc[tuvL(stuv[s0 + j])];
    }
    put4(Ah, Al, p, v);
  }
  if (arows > r8) clear_rows<NT>(Ah, Al, r8, arows, tid);
  arows = rows;
}

// Hermite indices of (s + n) for the four terms s0 .. s0+3 (s0 a multiple
// of 4) of one Hankel row n, from the table g_hx.
__device__ __forceinline__ uint2 hx4(int n, int s0) {
  return __ldg(reinterpret_cast<const uint2 *>(g_hx + n * NHS + s0));
}

// B rows of a Hankel matrix: row q < n1 (a multiple of 8), term s of the
// chunk: tab[(s+q) * tstride + toff] (zero beyond nR rows or nK terms).
template <int NT>
__device__ __forceinline__ void stage_hankel(float *Bh, float *Bl, const float *tab, int tstride,
                                             int toff, int n1, int nR, int kc, int nK,
                                             const uint32_t *stuv, int tid) {
  for (int p = tid; p < n1 * (KC / 4); p += NT) {
    int n = prow(p), s0 = kc + pk(p);
    float v[4] = {0.f, 0.f, 0.f, 0.f};
    if (n < nR) {
      uint2 w = hx4(n, s0);
      int ix[4] = {(int)(w.x & 0xFFFF), (int)(w.x >> 16), (int)(w.y & 0xFFFF), (int)(w.y >> 16)};
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (s0 + j < nK) v[j] = tab[ix[j] * tstride + toff];
    }
    put4(Bh, Bl, p, v);
  }
}

// The Hankel rows of the Breit kernel-table entries (i, j) for components
// i = ilo .. ilo+nb-1 (nb <= 3) at once, the table index of each element
// found once: entry (i, j) of the 6 symmetric ones (i for i = j, else
// i + j + 2) into the (i - ilo)-th B operand, hi at Bb + 2 (i - ilo) bstride
// and lo bstride floats after it.
template <int NT>
__device__ __forceinline__ void stage_hankel_n(float *Bb, int bstride, int ilo, int nb, int cj,
                                               const float *tab, int tstride, int n1, int nR,
                                               int kc, int nK, const uint32_t *stuv, int tid) {
  for (int p = tid; p < n1 * (KC / 4); p += NT) {
    int n = prow(p), s0 = kc + pk(p);
    int idx[4] = {-1, -1, -1, -1};
    if (n < nR) {
      uint2 w = hx4(n, s0);
      int ix[4] = {(int)(w.x & 0xFFFF), (int)(w.x >> 16), (int)(w.y & 0xFFFF), (int)(w.y >> 16)};
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (s0 + j < nK) idx[j] = ix[j] * tstride;
    }
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      if (b >= nb) break;
      float v[4];
      int ci = ilo + b, sw = ci == cj ? ci : ci + cj + 2;
#pragma unroll
      for (int j = 0; j < 4; ++j) v[j] = idx[j] >= 0 ? tab[idx[j] + sw] : 0.f;
      float *H = Bb + 2 * b * bstride;
      put4(H, H + bstride, p, v);
    }
  }
}

// A rows of GEMM 2 from D1 in tensor memory (TMEM address ta of column kc at
// lane 0): rows below `rows` only (D1's other rows are zero), each column q
// times sc[|q|] = (-1)^|q| 2^(kdiff |q|); warps sharing a lane quarter split
// the 32 columns.
template <int NT>
__device__ __forceinline__ void stage_g(float *Ah, float *Al, uint32_t ta, int kc, int nR,
                                        int rows, const float *sc, const uint32_t *stuv,
                                        int &arows, int warp, int lane, int tid) {
  constexpr int NQ = NT / 128, CW = KC / NQ;
  int quad = warp & 3, c0 = CW * (warp >> 2);
  int row = quad * 32 + lane;
  if (quad * 32 < rows) {  // warp-uniform: the TMEM load is warp-collective
    float v[CW];
    uint32_t a = ta + ((uint32_t)(quad * 32) << 16) + (uint32_t)c0;
    if (CW == 16) tld16(a, v); else tld8(a, v);
    if (row < rows) {
#pragma unroll
      for (int m = 0; m < CW / 4; ++m) {
        float x[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          int qq = kc + c0 + 4 * m + j;
          x[j] = qq < nR ? v[4 * m + j] * sc[tuvL(stuv[qq])] : 0.f;
        }
        put4(Ah, Al, piece(row, c0 + 4 * m), x);
      }
    }
  }
  if (arows > rows) clear_rows<NT>(Ah, Al, rows, arows, tid);
  arows = rows;
}

// B rows of GEMM 2 from the right pair's E-coefficients: row (label, set,
// re/im) for nlR labels, rows of (label, set) rstride apart; zero rows up
// to n2 (a multiple of 8).
template <int NT>
__device__ __forceinline__ void stage_er(float *Bh, float *Bl, const float2 *src,
                                         long long rstride, int nlR, int n2, int kc, int nR,
                                         int tid) {
  const int rows = 4 * nlR;
  const float *sf = reinterpret_cast<const float *>(src);
  for (int p = tid; p < n2 * (KC / 4); p += NT) {
    int row = prow(p), q0 = kc + pk(p);
    float v[4] = {0.f, 0.f, 0.f, 0.f};
    if (row < rows) {
      const float *e = sf + 2 * ((long long)(row >> 1) * rstride + q0) + (row & 1);
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (q0 + j < nR) v[j] = __ldg(e + 2 * j);
    }
    put4(Bh, Bl, p, v);
  }
}

// The 12 MMAs of one staged K chunk (4 steps of K = 8, three TF32 passes
// each) into the accumulator at TMEM address d; acc0 = 0 starts it.
__device__ __forceinline__ void issue_chunk(uint32_t d, const float *Ah, const float *Al,
                                            const float *Bh, const float *Bl, uint32_t id,
                                            bool acc0) {
#pragma unroll
  for (int ks = 0; ks < KC / 8; ++ks) {
    uint32_t off = ks * 256;
    uint64_t ah = sdesc(saddr(Ah) + off), al = sdesc(saddr(Al) + off);
    uint64_t bh = sdesc(saddr(Bh) + off), bl = sdesc(saddr(Bl) + off);
    mma(d, ah, bh, id, (acc0 || ks > 0) ? 1u : 0u);
    mma(d, ah, bl, id, 1u);
    mma(d, al, bh, id, 1u);
  }
}

// D2 columns c0 .. c0+ncol-1 of this thread's lane into the slab P (row
// stride PSTR), warps sharing a lane quarter taking 16-column pieces in turn.
template <int NT>
__device__ __forceinline__ void load_slab(float *P, uint32_t tD2, int c0, int ncol, int rows,
                                          int warp, int lane) {
  constexpr int NQ = NT / 128;
  int quad = warp & 3, row = quad * 32 + lane;
  if (quad * 32 >= rows) return;
  for (int j0 = 16 * (warp >> 2); j0 < ncol; j0 += 16 * NQ) {
    float v[16];
    tld16(tD2 + ((uint32_t)(quad * 32) << 16) + (uint32_t)(c0 + j0), v);
#pragma unroll
    for (int j = 0; j < 16; ++j) P[row * PSTR + j0 + j] = v[j];
  }
}

// FP64 R recursion (RMAKE's MD recursion, :31900) for one quartet into R/R2
// (level by level, one barrier per level); returns the buffer holding
// R^{(0)}.  G holds (-2 alpha)^n F_n for n = 0..lam (the k_qprep record),
// (X, Y, Z) = P - Q, dn[i] = i.
template <int NT>
__device__ __forceinline__ double *r_recursion(double *R, double *R2, const double *G, int lam,
                                               double X, double Y, double Z, const double *dn,
                                               const uint32_t *stuv, int tid) {
  double *cur = R, *nxt = R2;
  for (int n = lam; n >= 0; --n) {
    int cnt = ntuv(lam - n);
    for (int k = tid; k < cnt; k += NT) {
      double val;
      if (k == 0) {
        val = G[n];
      } else {
        uint32_t w = stuv[k];
        int t = w & 255, u = (w >> 8) & 255, v = (w >> 16) & 255;
        if (t > 0) {
          val = X * cur[hidx(t - 1, u, v)];
          if (t > 1) val += dn[t - 1] * cur[hidx(t - 2, u, v)];
        } else if (u > 0) {
          val = Y * cur[hidx(t, u - 1, v)];
          if (u > 1) val += dn[u - 1] * cur[hidx(t, u - 2, v)];
        } else {
          val = Z * cur[hidx(t, u, v - 1)];
          if (v > 1) val += dn[v - 1] * cur[hidx(t, u, v - 2)];
        }
      }
      nxt[k] = val;
    }
    __syncthreads();
    double *tmp = cur; cur = nxt; nxt = tmp;
  }
  return cur;
}

}  // namespace tcq

// ---------------------------------------------------------------------------
// Coulomb kernel
// ---------------------------------------------------------------------------
template <int NT, bool F64ACC>
__global__ void __launch_bounds__(NT, NT >= 512 ? 1 : 2)
k_quartet_tc(tcq::Args q, const int4 *quart, long long nq, int t1, int t2) {
  using namespace tcq;
  extern __shared__ unsigned char tc_smem_raw[];
  unsigned char *base =
      (unsigned char *)(((uintptr_t)tc_smem_raw + 127) & ~(uintptr_t)127);
  // shared J/K accumulators: FP64 in Fock builds (repeated builds agree to
  // FP64 rounding, which an SCF needs), FP32 for one-shot explicit lists
  using Acc2 = typename std::conditional<F64ACC, double2, float2>::type;
  using AccS = typename std::conditional<F64ACC, double, float>::type;
  const Layout LY = layout_c(q.n1max, q.n2max, q.nbuf, F64ACC);
  const int bmax = q.n1max > q.n2max ? q.n1max : q.n2max;
  auto bufA = [&](int b) { return (float *)(base + LY.abuf + b * ABYTES); };
  auto bufB = [&](int b) { return (float *)(base + LY.bbuf + b * LY.bsz); };
  float *P = (float *)(base + LY.bbuf);           // D2 slab (epilogue)
  double *R = (double *)(base + LY.bbuf);         // FP64 recursion (before the GEMMs)
  double *R2 = R + NTR;
  float *Rf = (float *)(base + LY.rf);
  float2 *Dsm = (float2 *)(base + LY.dsm);        // D(c,d), D(c,b), D(a,b), D(a,d)
  Acc2 *Acc = (Acc2 *)(base + LY.acc);            // J(a,b), K(a,d), J2(c,d), K2(c,b)
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t tslot;
  __shared__ double sqp[QPW];          // this quartet's k_qprep record
  __shared__ double spre[MAXLAM + 1];  // PRE 2^(-k lambda)
  __shared__ double sdn[MAXLAM + 1];   // sdn[i] = i
  __shared__ float sEs[MAXDEGE + 1], sGs[MAXDEGE + 1];  // staging scales per lambda
  __shared__ uint32_t stuv[NTR];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nbuf = q.nbuf;

  for (int i = tid; i <= MAXLAM; i += NT) sdn[i] = (double)i;
  for (int i = tid; i < NTR; i += NT)
    stuv[i] = (uint32_t)c_t[i] | ((uint32_t)c_u[i] << 8) | ((uint32_t)c_v[i] << 16) |
              ((uint32_t)(c_t[i] + c_u[i] + c_v[i]) << 24);
  for (int i = tid; i < nbuf * 2 * MROWS * KC; i += NT) bufA(0)[i] = 0.f;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(saddr(&tslot)), "r"(q.tmem_cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(saddr(&mbar[0])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(saddr(&mbar[1])));
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tslot;
  Pipe pp = {mbar, {0u, 0u}, {false, false}};
  int arows[2] = {0, 0};  // rows of each A buffer that may be nonzero
  bool abort = false;
  // the next quartet's record is loaded while this one is digested
  double qnext = (tid < QPW && blockIdx.x < nq) ? q.qp[blockIdx.x * (long long)QPW + tid] : 0.0;

  for (long long qi = blockIdx.x; qi < nq && !abort; qi += gridDim.x) {
    const double qcur = qnext;
    if (tid < QPW && qi + gridDim.x < nq) qnext = q.qp[(qi + gridDim.x) * QPW + tid];
    int4 Q4 = quart[qi];
    const Shell &A = q.sh[Q4.x], &B = q.sh[Q4.y], &C = q.sh[Q4.z], &Dd = q.sh[Q4.w];
    int la = A.l, lb = B.l, lc = C.l, ld = Dd.l;
    int degab = la + lb + 2 * t1, degcd = lc + ld + 2 * t2;
    int lam = degab + degcd;
    int nla = 2 * la + 1, nlb = 2 * lb + 1, nlc = 2 * lc + 1, nld = 2 * ld + 1;
    int nab = ntuv(degab), ncd = ntuv(degcd);
    int n1, n2;
    bool swp;
    tc_dims(la, lb, lc, ld, t1, t2, n1, n2, swp);
    if (n1 + n2 > q.tmem_cols || n1 > q.n1max || n2 > q.n2max) {
      if (tid == 0) atomicOr(&g_tc_status, 2);  // launch sized for other classes
      continue;
    }
    int mcnt = ncntrs(A.cnt, B.cnt, C.cnt, Dd.cnt);
    const double2 *Dm = q.D;
    double *GDm = q.GD, *GXm = q.GX;
    size_t lddm = q.ldd, ldfm = q.ldf;
    int nskpm = q.nskp;
    if (q.inst) {
      const Inst I = q.inst[A.inst];
      Dm += I.off;
      GDm += 2 * I.off;
      GXm += 2 * I.off;
      lddm = ldfm = (size_t)I.ld;
      nskpm = I.nskp;
    }
    const PairE &pab_e = q.pe[A.prow + Q4.y], &pcd_e = q.pe[C.prow + Q4.w];
    // the previous quartet's reads of sqp ended before its GEMMs' barriers
    if (tid < QPW) sqp[tid] = qcur;
    // the previous quartet's TMEM reads and shared-memory use end here
    fence_before();
    __syncthreads();
    fence_after();
    const int kq0 = (int)sqp[7];  // exponent-balancing shift k
    if (tid <= lam) spre[tid] = ldexp(sqp[4], -kq0 * tid);
    {
      // R with P - Q in the orientation the contractions take
      double sg = swp ? -1.0 : 1.0;
      const double *cur = r_recursion<NT>(R, R2, sqp + 8, lam, sg * sqp[0], sg * sqp[1],
                                          sg * sqp[2], sdn, stuv, tid);
      // PRE * R scaled by 2^(-k lambda) (exponent balancing), in FP32
      for (int i = tid; i < ntuv(lam); i += NT)
        Rf[i] = __double2float_rn(cur[i] * spre[tuvL(stuv[i])]);
    }
    // roles
    const float2 *Eab = q.E + pab_e.off[t1];
    const float2 *Ecd = q.E + pcd_e.off[t2];
    const float2 *EL = swp ? Ecd : Eab, *ER = swp ? Eab : Ecd;
    int kL = swp ? pcd_e.kexp : pab_e.kexp, kR = swp ? pab_e.kexp : pcd_e.kexp;
    int nL = swp ? ncd : nab, nR = swp ? nab : ncd;
    int nlab = nla * nlb, nlcd = nlc * nld;
    int nlL = swp ? nlcd : nlab, nlR = swp ? nlab : nlcd;
    int nl2L = swp ? nld : nlb, nl2R = swp ? nlb : nld;
    int lq[4] = {la, lb, lc, ld};
    int oab = t1 ? nskpm : 0, ocd = t2 ? nskpm : 0;
    if (tid <= MAXDEGE) {
      sEs[tid] = ldexpf(1.0f, (kq0 - kL) * tid);
      sGs[tid] = ldexpf((tid & 1) ? -1.0f : 1.0f, (kq0 - kR) * tid);
    }
    bool dual = q.sym && (Q4.x != Q4.z || Q4.y != Q4.w || t1 != t2);
    // density blocks of this quartet: D(c,d), D(c,b), and for (cd|ab) D(a,b), D(a,d)
    {
      int sizes[4][2] = {{2 * nlc, 2 * nld}, {2 * nlc, 2 * nlb}, {2 * nla, 2 * nlb},
                         {2 * nla, 2 * nld}};
      const Shell *rs[4] = {&C, &C, &A, &A}, *cs[4] = {&Dd, &B, &B, &Dd};
      int ro[4] = {ocd, ocd, oab, oab}, co[4] = {ocd, oab, oab, ocd};
      for (int blk = 0; blk < (dual ? 4 : 2); ++blk) {
        int nr = sizes[blk][0], nc = sizes[blk][1];
        for (int w = tid; w < nr * nc; w += NT) {
          int r = w / nc, c = w % nc;
          int fr = rs[blk]->fock[r >> 1][r & 1] + ro[blk];
          int fc = cs[blk]->fock[c >> 1][c & 1] + co[blk];
          double2 v = Dm[(size_t)fr + lddm * fc];
          Dsm[blk * MAXSP * MAXSP + r * MAXSP + c] =
              make_float2(__double2float_rn(v.x), __double2float_rn(v.y));
        }
      }
    }
    for (int i = tid; i < 4 * MAXSP * MAXSP; i += NT) {
      Acc[i].x = AccS(0);
      Acc[i].y = AccS(0);
    }
    __syncthreads();  // R (FP64) is dead: the B buffers may overwrite it

    const uint32_t tD1 = tmem, tD2 = tmem + (uint32_t)n1;
    const uint32_t id1 = idesc(MROWS, n1), id2 = idesc(MROWS, n2);
    for (int l0 = 0; l0 < nlL && !abort; l0 += MLAB) {
      int ntl = min(MLAB, nlL - l0), rows = 4 * ntl;
      // ---- GEMM 1: D1 = E_L (rows) x Hankel R (columns q), K = s ----
      // K chunk c is staged into buffer c % nbuf while the MMAs of chunk
      // c - 1 run; a buffer is rewritten once its previous MMAs completed
      for (int c = 0, kc = 0; kc < nL && !abort; ++c, kc += KC) {
        int bsel = c % nbuf;
        if (__syncthreads_or(!pipe_wait(pp, bsel))) { abort = true; break; }
        fence_after();
        float *Ah = bufA(bsel), *Al = Ah + MROWS * KC;
        float *Bh = bufB(bsel), *Bl = Bh + bmax * KC;
        stage_e_rows<NT>(Ah, Al, EL + (long long)l0 * 2 * nL, nL, ntl, kc, nL, sEs, stuv,
                         arows[bsel], tid);
        stage_hankel<NT>(Bh, Bl, Rf, 1, 0, n1, nR, kc, nL, stuv, tid);
        fence_async_smem();
        fence_before();
        __syncthreads();
        if (tid == 0) {
          fence_after();
          issue_chunk(tD1, Ah, Al, Bh, Bl, id1, kc > 0);
          commit(&pp.bar[bsel]);
        }
        pp.pend[bsel] = true;
      }
      // D1 complete before its columns are read
      {
        bool ok = pipe_wait(pp, 0);
        ok = pipe_wait(pp, 1) && ok;
        if (__syncthreads_or(!ok)) abort = true;
        fence_after();
      }
      // ---- GEMM 2: D2 = G (rows, K = q) x E_R (columns) ----
      for (int c = 0, kc = 0; kc < n1 && !abort; ++c, kc += KC) {
        int bsel = c % nbuf;
        if (__syncthreads_or(!pipe_wait(pp, bsel))) { abort = true; break; }
        fence_after();
        float *Ah = bufA(bsel), *Al = Ah + MROWS * KC;
        float *Bh = bufB(bsel), *Bl = Bh + bmax * KC;
        stage_g<NT>(Ah, Al, tD1 + (uint32_t)kc, kc, nR, rows, sGs, stuv, arows[bsel], warp,
                    lane, tid);
        stage_er<NT>(Bh, Bl, ER, nR, nlR, n2, kc, nR, tid);
        fence_async_smem();
        fence_before();
        __syncthreads();
        if (tid == 0) {
          fence_after();
          issue_chunk(tD2, Ah, Al, Bh, Bl, id2, kc > 0);
          commit(&pp.bar[bsel]);
        }
        pp.pend[bsel] = true;
      }
      {
        bool ok = pipe_wait(pp, 0);
        ok = pipe_wait(pp, 1) && ok;
        if (__syncthreads_or(!ok)) abort = true;
        fence_after();
      }
      if (abort) break;
      // ---- epilogue: 16 products per label pair -> m-sign combinations ->
      //      J/K digestion (FP32 products, per-quartet FP32 sums) ----
      for (int c0 = 0; c0 < 4 * nlR; c0 += SLAB) {
        int ncol = min(SLAB, n2 - c0);
        load_slab<NT>(P, tD2, c0, ncol, rows, warp, lane);
        fence_before();
        __syncthreads();
        int r0 = c0 / 4, nrl = min(SLAB / 4, nlR - r0);
        for (int w = tid; w < ntl * nrl; w += NT) {
          int lab = w % ntl;
          int lr = r0 + (w / ntl + lab) % nrl;  // skewed: lanes hit different targets
          int labL = l0 + lab;
          int l1 = labL / nl2L, l2 = labL % nl2L, r1 = lr / nl2R, r2 = lr % nl2R;
          int ia = swp ? r1 : l1, ib = swp ? r2 : l2, ic = swp ? l1 : r1, id = swp ? l2 : r2;
          int kq[4], mq[4], mm[4];
          label_of(la, ia, kq[0], mm[0]);
          label_of(lb, ib, kq[1], mm[1]);
          label_of(lc, ic, kq[2], mm[2]);
          label_of(ld, id, kq[3], mm[3]);
          for (int i = 0; i < 4; ++i) mq[i] = 2 * mm[i] - 1;
          if (!label_ok(q.isym, q.racah1, mcnt, kq, mq, lq)) continue;
          float2 sv[8];
          products8(P + (lab * 4) * PSTR + (lr - r0) * 4, sv);
          double pab = pair_phase(kq[0], mm[0], kq[1], mm[1]);
          double pcd = pair_phase(kq[2], mm[2], kq[3], mm[3]);
          double pl = swp ? pcd : pab, pr = swp ? pab : pcd;
          float sl = pl < 0 ? -1.f : 1.f, slr = (pl * pr) < 0 ? -1.f : 1.f;
          const float2 *Dcd = Dsm, *Dcb = Dsm + MAXSP * MAXSP;
          const float2 *Dab = Dsm + 2 * MAXSP * MAXSP, *Dad = Dsm + 3 * MAXSP * MAXSP;
          Acc2 *Jl = Acc, *Kl = Acc + MAXSP * MAXSP, *J2 = Acc + 2 * MAXSP * MAXSP,
               *K2 = Acc + 3 * MAXSP * MAXSP;
          float2 r16[16];
          combos16(sv, sl, slr, r16);
          // (ab|cd) m-sign combination from the (left|right) one; every index
          // is a compile-time constant once the loops are unrolled
#define TCV(sa, sb, sc, sd) (swp ? r16[8 * (sc) + 4 * (sd) + 2 * (sa) + (sb)] \
                                 : r16[8 * (sa) + 4 * (sb) + 2 * (sc) + (sd)])
          if (q.isym == 0) {
#pragma unroll
            for (int sa = 0; sa < 2; ++sa)
#pragma unroll
              for (int sb = 0; sb < 2; ++sb) {
                float2 j = make_float2(0.f, 0.f);
#pragma unroll
                for (int sc = 0; sc < 2; ++sc)
#pragma unroll
                  for (int sd = 0; sd < 2; ++sd)
                    cmac(j, TCV(sa, sb, sc, sd), Dcd[(ic * 2 + sc) * MAXSP + id * 2 + sd]);
                sadd(&Jl[(ia * 2 + sa) * MAXSP + ib * 2 + sb], j);
              }
#pragma unroll
            for (int sa = 0; sa < 2; ++sa)
#pragma unroll
              for (int sd = 0; sd < 2; ++sd) {
                float2 k = make_float2(0.f, 0.f);
#pragma unroll
                for (int sb = 0; sb < 2; ++sb)
#pragma unroll
                  for (int sc = 0; sc < 2; ++sc)
                    cmac(k, TCV(sa, sb, sc, sd), Dcb[(ic * 2 + sc) * MAXSP + ib * 2 + sb]);
                sadd(&Kl[(ia * 2 + sa) * MAXSP + id * 2 + sd], k);
              }
            if (dual) {
#pragma unroll
              for (int sc = 0; sc < 2; ++sc)
#pragma unroll
                for (int sd = 0; sd < 2; ++sd) {
                  float2 j = make_float2(0.f, 0.f);
#pragma unroll
                  for (int sa = 0; sa < 2; ++sa)
#pragma unroll
                    for (int sb = 0; sb < 2; ++sb)
                      cmac(j, TCV(sa, sb, sc, sd), Dab[(ia * 2 + sa) * MAXSP + ib * 2 + sb]);
                  sadd(&J2[(ic * 2 + sc) * MAXSP + id * 2 + sd], j);
                }
#pragma unroll
              for (int sc = 0; sc < 2; ++sc)
#pragma unroll
                for (int sb = 0; sb < 2; ++sb) {
                  float2 k = make_float2(0.f, 0.f);
#pragma unroll
                  for (int sa = 0; sa < 2; ++sa)
#pragma unroll
                    for (int sd = 0; sd < 2; ++sd)
                      cmac(k, TCV(sa, sb, sc, sd), Dad[(ia * 2 + sa) * MAXSP + id * 2 + sd]);
                  sadd(&K2[(ic * 2 + sc) * MAXSP + ib * 2 + sb], k);
                }
            }
          } else {
            // CLMMTZ: real parts, equal-sign direct blocks, crossed exchange
#pragma unroll
            for (int s = 0; s < 2; ++s) {
              float jv = 0.f, kv = 0.f;
#pragma unroll
              for (int t = 0; t < 2; ++t) {
                jv = fmaf(TCV(s, s, t, t).x, Dcd[(ic * 2 + t) * MAXSP + id * 2 + t].x, jv);
                kv = fmaf(TCV(s, t, t, s).x, Dcb[(ic * 2 + t) * MAXSP + ib * 2 + t].x, kv);
              }
              atomicAdd(&Jl[(ia * 2 + s) * MAXSP + ib * 2 + s].x, (AccS)jv);
              atomicAdd(&Kl[(ia * 2 + s) * MAXSP + id * 2 + s].x, (AccS)kv);
            }
            if (dual) {
#pragma unroll
              for (int s = 0; s < 2; ++s) {
                float jv = 0.f, kv = 0.f;
#pragma unroll
                for (int t = 0; t < 2; ++t) {
                  jv = fmaf(TCV(t, t, s, s).x, Dab[(ia * 2 + t) * MAXSP + ib * 2 + t].x, jv);
                  kv = fmaf(TCV(t, s, s, t).x, Dad[(ia * 2 + t) * MAXSP + id * 2 + t].x, kv);
                }
                atomicAdd(&J2[(ic * 2 + s) * MAXSP + id * 2 + s].x, (AccS)jv);
                atomicAdd(&K2[(ic * 2 + s) * MAXSP + ib * 2 + s].x, (AccS)kv);
              }
            }
          }
#undef TCV
        }
        __syncthreads();  // the slab buffer is rewritten next
      }
    }
    if (abort) break;
    // flush: weight 1/2 for a quartet equal to its (ba|dc) image, or to its
    // (dc|ba) image within one class; FP64 accumulation in global memory
    const double wq = (q.sym == 2 && ((Q4.x == Q4.y && Q4.z == Q4.w) ||
                                      (t1 == t2 && Q4.x == Q4.w && Q4.y == Q4.z))) ? 0.5 : 1.0;
    const int rr[4][2] = {{0, 1}, {0, 3}, {2, 3}, {2, 1}};  // roles (row, column) per target
    const Shell *sh4[4] = {&A, &B, &C, &Dd};
    const int nl4[4] = {nla, nlb, nlc, nld}, off4[4] = {oab, oab, ocd, ocd};
    for (int f = 0; f < (dual ? 4 : 2); ++f) {
      int ra = rr[f][0], ca = rr[f][1];
      int nr = 2 * nl4[ra], nc = 2 * nl4[ca];
      double *G = (f == 0 || f == 2) ? GDm : GXm;
      for (int w = tid; w < nr * nc; w += NT) {
        int a = w / nc, b = w % nc;
        Acc2 v = Acc[f * MAXSP * MAXSP + a * MAXSP + b];
        if (v.x == AccS(0) && v.y == AccS(0)) continue;
        int fa = sh4[ra]->fock[a >> 1][a & 1] + off4[ra];
        int fb = sh4[ca]->fock[b >> 1][b & 1] + off4[ca];
        double *dst = G + 2 * ((size_t)fa + ldfm * fb);
        atomicAdd(dst, wq * (double)v.x);
        atomicAdd(dst + 1, wq * (double)v.y);
      }
    }
  }
  if (abort && tid == 0) atomicOr(&g_tc_status, 1);
  // release: every TMEM read and MMA of this CTA has completed (waited above;
  // after a timeout, wait once more, bounded, for the MMAs in flight)
  if (abort) {
    pipe_wait(pp, 0);
    pipe_wait(pp, 1);
  }
  fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                 :: "r"(tmem), "r"(q.tmem_cols));
}

// ---------------------------------------------------------------------------
// Tensor-core Breit kernel: BIIFAST's contractions (bertha-scf.f:18337-19171)
// on tcgen05 in the same 3xTF32 form.  With the 3x3 Breit kernel table
// W_ij(N) (Gaunt and gauge terms, :18655-18880; symmetric, 6 entries per N),
// per Cartesian component i of the right electron:
//   GEMM 1  D1_i[row][q]  = sum_j sum_s E_L[row][j][s] W_ij(s+q)
//   GEMM 2  D2[row][col] += sum_q G_i[row][q] E_R[col][i][q]
// D2 summed over i holds the 16 products per label pair; exchange digestion
// (BRTMTG/BRTMTZ batch type 5) with the Breit phases follows in FP32.  When
// three D1 fit in tensor memory beside D2 (tri), each staged E_L chunk feeds
// all three components at once; otherwise the components run one after the
// other.
// ---------------------------------------------------------------------------
template <int NT>
__global__ void __launch_bounds__(NT, NT >= 512 ? 1 : 2)
k_breit_tc(tcq::ArgsB q, const int4 *quart, long long nq, int t1, int t2) {
  using namespace tcq;
  extern __shared__ unsigned char tc_smem_raw[];
  unsigned char *base =
      (unsigned char *)(((uintptr_t)tc_smem_raw + 127) & ~(uintptr_t)127);
  const Layout LY = layout_b(q.n1max, q.n2max, q.nbuf, q.tri);
  auto bufA = [&](int b) { return (float *)(base + LY.abuf + b * ABYTES); };
  auto bufB = [&](int b) { return (float *)(base + LY.bbuf + b * LY.bsz); };
  float *P = (float *)(base + LY.bbuf);
  double *R = (double *)(base + LY.bbuf);
  double *R2 = R + NTR;
  float *Wf = (float *)(base + LY.rf);
  float2 *Dsm = (float2 *)(base + LY.dsm);   // D(c,b), D(a,d)
  double2 *Acc = (double2 *)(base + LY.acc); // K(a,d), K2(c,b)
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t tslot;
  __shared__ double sqp[QPW];          // this quartet's k_qprep record
  __shared__ double s2k[MAXLAM + 1];   // 2^(-k lambda)
  __shared__ double sdn[MAXLAM + 1];   // sdn[i] = i
  __shared__ float sEs[MAXDEGE + 1], sGs[MAXDEGE + 1];  // staging scales per lambda
  __shared__ uint32_t stuv[NTR];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nbuf = q.nbuf;

  for (int i = tid; i <= MAXLAM; i += NT) sdn[i] = (double)i;
  for (int i = tid; i < NTR; i += NT)
    stuv[i] = (uint32_t)c_t[i] | ((uint32_t)c_u[i] << 8) | ((uint32_t)c_v[i] << 16) |
              ((uint32_t)(c_t[i] + c_u[i] + c_v[i]) << 24);
  for (int i = tid; i < nbuf * 2 * MROWS * KC; i += NT) bufA(0)[i] = 0.f;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(saddr(&tslot)), "r"(q.tmem_cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(saddr(&mbar[0])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(saddr(&mbar[1])));
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tslot;
  Pipe pp = {mbar, {0u, 0u}, {false, false}};
  int arows[2] = {0, 0};
  bool abort = false;
  // the next quartet's record is loaded while this one is digested
  double qnext = (tid < QPW && blockIdx.x < nq) ? q.qp[blockIdx.x * (long long)QPW + tid] : 0.0;

  for (long long qi = blockIdx.x; qi < nq && !abort; qi += gridDim.x) {
    const double qcur = qnext;
    if (tid < QPW && qi + gridDim.x < nq) qnext = q.qp[(qi + gridDim.x) * QPW + tid];
    int4 Q4 = quart[qi];
    const Shell &A = q.sh[Q4.x], &B = q.sh[Q4.y], &C = q.sh[Q4.z], &Dd = q.sh[Q4.w];
    int la = A.l, lb = B.l, lc = C.l, ld = Dd.l;
    int degab = la + lb + 1, degcd = lc + ld + 1;
    int lamn = degab + degcd, lam = lamn + (q.gaunt ? 0 : 2);
    int nla = 2 * la + 1, nlb = 2 * lb + 1, nlc = 2 * lc + 1, nld = 2 * ld + 1;
    int nab = ntuv(degab), ncd = ntuv(degcd);
    int n1, n2;
    bool swp;
    tcb_dims(la, lb, lc, ld, q.gaunt, n1, n2, swp);
    if ((q.tri ? 3 * n1 : n1) + n2 > q.tmem_cols || n1 > q.n1max || n2 > q.n2max) {
      if (tid == 0) atomicOr(&g_tc_status, 2);
      continue;
    }
    int mcnt = ncntrs(A.cnt, B.cnt, C.cnt, Dd.cnt);
    bool dual = q.dual && (Q4.x != Q4.z || Q4.y != Q4.w || t1 != t2);
    // the previous quartet's reads of sqp ended before its GEMMs' barriers
    if (tid < QPW) sqp[tid] = qcur;
    fence_before();
    __syncthreads();
    fence_after();
    const int kq0 = (int)sqp[7];  // exponent-balancing shift k
    if (tid <= lamn) s2k[tid] = ldexp(1.0, -kq0 * tid);
    {
      // R and the kernel table for the left pair's centre minus the right's
      double sg = swp ? -1.0 : 1.0;
      const double *cur = r_recursion<NT>(R, R2, sqp + 8, lam, sg * sqp[0], sg * sqp[1],
                                          sg * sqp[2], sdn, stuv, tid);
      // kernel table W_ij(N) = BFAC (delta_ij R_N - T_ij(N)) from PRE * R,
      // scaled by 2^(-k lambda_N), FP32 (6 symmetric entries per N)
      double pre = sqp[4], h2a = sqp[6];
      double bfac = q.gaunt ? -1.0 : -0.5;
      for (int w = tid; w < ntuv(lamn) * 6; w += NT) {
        int n = w / 6, e = w % 6;
        int i = e < 3 ? e : (e == 5 ? 1 : 0), j = e < 3 ? e : (e == 3 ? 1 : 2);
        uint32_t tw = stuv[n];
        int N0 = (int)(tw & 255), N1 = (int)((tw >> 8) & 255), N2 = (int)((tw >> 16) & 255);
        double rn = cur[n] * pre;
        double val;
        if (q.gaunt) {
          val = i == j ? -rn : 0.0;
        } else {
          // a = N + e_i + e_j, then a - e_j, then a - 2 e_j
          int a0 = N0 + (i == 0) + (j == 0), a1 = N1 + (i == 1) + (j == 1);
          int a2 = N2 + (i == 2) + (j == 2);
          double tt = cur[hidx(a0, a1, a2)] * h2a;
          a0 -= j == 0; a1 -= j == 1; a2 -= j == 2;
          double pqj = -sg * sqp[j];  // (Q - P)_j in the orientation taken
          tt -= cur[hidx(a0, a1, a2)] * pqj;
          a0 -= j == 0; a1 -= j == 1; a2 -= j == 2;
          int aj = j == 0 ? a0 : (j == 1 ? a1 : a2), Nj = j == 0 ? N0 : (j == 1 ? N1 : N2);
          if (aj >= 0) tt += cur[hidx(a0, a1, a2)] * sdn[Nj];
          val = bfac * ((i == j ? rn : 0.0) - tt * pre);
        }
        Wf[w] = __double2float_rn(val * s2k[tuvL(tw)]);
      }
    }
    const PairE &pab_e = q.pe[A.prow + Q4.y], &pcd_e = q.pe[C.prow + Q4.w];
    const float2 *Eab = q.E + q.offq[((size_t)Q4.x * q.ns + Q4.y) * 2 + t1];
    const float2 *Ecd = q.E + q.offq[((size_t)Q4.z * q.ns + Q4.w) * 2 + t2];
    const float2 *EL = swp ? Ecd : Eab, *ER = swp ? Eab : Ecd;
    int kL = swp ? pcd_e.kexp : pab_e.kexp, kR = swp ? pab_e.kexp : pcd_e.kexp;
    int nL = swp ? ncd : nab, nR = swp ? nab : ncd;
    int nlab = nla * nlb, nlcd = nlc * nld;
    int nlL = swp ? nlcd : nlab, nlR = swp ? nlab : nlcd;
    int nl2L = swp ? nld : nlb, nl2R = swp ? nlb : nld;
    int lq[4] = {la, lb, lc, ld};
    // Fock offsets: an LS pair has its first function large, second small
    int oa = t1 ? q.nskp : 0, ob = t1 ? 0 : q.nskp;
    int oc = t2 ? q.nskp : 0, od = t2 ? 0 : q.nskp;
    if (tid <= MAXDEGE) {
      sEs[tid] = ldexpf(1.0f, (kq0 - kL) * tid);
      sGs[tid] = ldexpf((tid & 1) ? -1.0f : 1.0f, (kq0 - kR) * tid);
    }
    {
      // D(c,b) and, for (cd|ab), D(a,d)
      int sizes[2][2] = {{2 * nlc, 2 * nlb}, {2 * nla, 2 * nld}};
      const Shell *rs[2] = {&C, &A}, *cs[2] = {&B, &Dd};
      int ro[2] = {oc, oa}, co[2] = {ob, od};
      for (int blk = 0; blk < (dual ? 2 : 1); ++blk) {
        int nr = sizes[blk][0], nc = sizes[blk][1];
        for (int w = tid; w < nr * nc; w += NT) {
          int r = w / nc, c = w % nc;
          int fr = rs[blk]->fock[r >> 1][r & 1] + ro[blk];
          int fc = cs[blk]->fock[c >> 1][c & 1] + co[blk];
          double2 v = q.D[(size_t)fr + (size_t)q.ldd * fc];
          Dsm[blk * MAXSP * MAXSP + r * MAXSP + c] =
              make_float2(__double2float_rn(v.x), __double2float_rn(v.y));
        }
      }
    }
    for (int i = tid; i < 2 * MAXSP * MAXSP; i += NT) Acc[i] = make_double2(0.0, 0.0);
    __syncthreads();

    const int nslot = q.tri ? 3 : 1;  // D1 accumulators side by side
    const uint32_t tD2 = tmem + (uint32_t)(nslot * n1);
    const uint32_t id1 = idesc(MROWS, n1), id2 = idesc(MROWS, n2);
    const long long rsL = 3LL * nL, rsR = 3LL * nR;  // (label, set) strides of the E blocks
    for (int l0 = 0; l0 < nlL && !abort; l0 += MLAB) {
      int ntl = min(MLAB, nlL - l0), rows = 4 * ntl;
      const float2 *ELt = EL + (long long)l0 * 2 * rsL;
      int c = 0;  // chunk counter (buffer selection) across the passes
      // passes: all three components at once (tri), or one after the other
      for (int i0 = 0; i0 < 3 && !abort; i0 += nslot) {
        int i1 = i0 + nslot;
        // ---- GEMM 1: D1_i for i0 <= i < i1, K over (j, s) ----
        for (int cj = 0; cj < 3 && !abort; ++cj) {
          // components i of this pass that couple to j (Gaunt: i = j only)
          int ilo = q.gaunt ? cj : i0, ihi = q.gaunt ? cj + 1 : i1;
          if (ilo < i0) ilo = i0;
          if (ihi > i1) ihi = i1;
          if (ilo >= ihi) continue;
          for (int kc = 0; kc < nL && !abort; kc += KC, ++c) {
            int bsel = c % nbuf;
            if (__syncthreads_or(!pipe_wait(pp, bsel))) { abort = true; break; }
            fence_after();
            float *Ah = bufA(bsel), *Al = Ah + MROWS * KC;
            float *Bb = bufB(bsel);
            stage_e_rows<NT>(Ah, Al, ELt + (long long)cj * nL, rsL, ntl, kc, nL, sEs, stuv,
                             arows[bsel], tid);
            stage_hankel_n<NT>(Bb + (ilo - i0) * 2 * q.n1max * KC, q.n1max * KC, ilo, ihi - ilo,
                               cj, Wf, 6, n1, nR, kc, nL, stuv, tid);
            fence_async_smem();
            fence_before();
            __syncthreads();
            if (tid == 0) {
              fence_after();
              for (int ci = ilo; ci < ihi; ++ci) {
                float *Bh = Bb + (ci - i0) * 2 * q.n1max * KC, *Bl = Bh + q.n1max * KC;
                // first contribution to D1_i: j = 0 (Gaunt: j = i) at kc = 0
                bool acc0 = kc > 0 || (!q.gaunt && cj > 0);
                issue_chunk(tmem + (uint32_t)((ci - i0) * n1), Ah, Al, Bh, Bl, id1, acc0);
              }
              commit(&pp.bar[bsel]);
            }
            pp.pend[bsel] = true;
          }
        }
        {
          bool ok = pipe_wait(pp, 0);
          ok = pipe_wait(pp, 1) && ok;
          if (__syncthreads_or(!ok)) abort = true;
          fence_after();
        }
        // ---- GEMM 2 for the pass's components, accumulated over i ----
        for (int ci = i0; ci < i1 && !abort; ++ci) {
          uint32_t tD1 = tmem + (uint32_t)((ci - i0) * n1);
          for (int kc = 0; kc < n1 && !abort; kc += KC, ++c) {
            int bsel = c % nbuf;
            if (__syncthreads_or(!pipe_wait(pp, bsel))) { abort = true; break; }
            fence_after();
            float *Ah = bufA(bsel), *Al = Ah + MROWS * KC;
            float *Bh = bufB(bsel), *Bl = Bh + q.n2max * KC;
            stage_g<NT>(Ah, Al, tD1 + (uint32_t)kc, kc, nR, rows, sGs, stuv, arows[bsel],
                        warp, lane, tid);
            stage_er<NT>(Bh, Bl, ER + (long long)ci * nR, rsR, nlR, n2, kc, nR, tid);
            fence_async_smem();
            fence_before();
            __syncthreads();
            if (tid == 0) {
              fence_after();
              issue_chunk(tD2, Ah, Al, Bh, Bl, id2, ci > 0 || kc > 0);
              commit(&pp.bar[bsel]);
            }
            pp.pend[bsel] = true;
          }
        }
        {
          // D1 is rewritten by the next pass, D2 read by the epilogue
          bool ok = pipe_wait(pp, 0);
          ok = pipe_wait(pp, 1) && ok;
          if (__syncthreads_or(!ok)) abort = true;
          fence_after();
        }
      }
      if (abort) break;
      // ---- epilogue: exchange digestion with the Breit phases ----
      for (int c0 = 0; c0 < 4 * nlR; c0 += SLAB) {
        int ncol = min(SLAB, n2 - c0);
        load_slab<NT>(P, tD2, c0, ncol, rows, warp, lane);
        fence_before();
        __syncthreads();
        int r0 = c0 / 4, nrl = min(SLAB / 4, nlR - r0);
        for (int w = tid; w < ntl * nrl; w += NT) {
          int lab = w % ntl;
          int lr = r0 + (w / ntl + lab) % nrl;
          int labL = l0 + lab;
          int l1 = labL / nl2L, l2 = labL % nl2L, r1 = lr / nl2R, r2 = lr % nl2R;
          int ia = swp ? r1 : l1, ib = swp ? r2 : l2, ic = swp ? l1 : r1, id = swp ? l2 : r2;
          int kq[4], mq[4], mm[4];
          label_of(la, ia, kq[0], mm[0]);
          label_of(lb, ib, kq[1], mm[1]);
          label_of(lc, ic, kq[2], mm[2]);
          label_of(ld, id, kq[3], mm[3]);
          for (int i = 0; i < 4; ++i) mq[i] = 2 * mm[i] - 1;
          if (!label_ok(q.isym, q.racah1, mcnt, kq, mq, lq, true)) continue;
          float2 sv[8];
          products8(P + (lab * 4) * PSTR + (lr - r0) * 4, sv);
          // Breit phases: the Coulomb pair phases negated (BRTFAST :17528-17533)
          double pab = -pair_phase(kq[0], mm[0], kq[1], mm[1]);
          double pcd = -pair_phase(kq[2], mm[2], kq[3], mm[3]);
          double pl = swp ? pcd : pab, pr = swp ? pab : pcd;
          float sl = pl < 0 ? -1.f : 1.f, slr = (pl * pr) < 0 ? -1.f : 1.f;
          const float2 *Dcb = Dsm, *Dad = Dsm + MAXSP * MAXSP;
          double2 *Kl = Acc, *K2 = Acc + MAXSP * MAXSP;
          float2 r16[16];
          combos16(sv, sl, slr, r16);
#define TCV(sa, sb, sc, sd) (swp ? r16[8 * (sc) + 4 * (sd) + 2 * (sa) + (sb)] \
                                 : r16[8 * (sa) + 4 * (sb) + 2 * (sc) + (sd)])
          if (q.isym == 0) {
#pragma unroll
            for (int sa = 0; sa < 2; ++sa)
#pragma unroll
              for (int sd = 0; sd < 2; ++sd) {
                float2 k = make_float2(0.f, 0.f);
#pragma unroll
                for (int sb = 0; sb < 2; ++sb)
#pragma unroll
                  for (int sc = 0; sc < 2; ++sc)
                    cmac(k, TCV(sa, sb, sc, sd), Dcb[(ic * 2 + sc) * MAXSP + ib * 2 + sb]);
                sadd(&Kl[(ia * 2 + sa) * MAXSP + id * 2 + sd], k);
              }
            if (dual) {
#pragma unroll
              for (int sc = 0; sc < 2; ++sc)
#pragma unroll
                for (int sb = 0; sb < 2; ++sb) {
                  float2 k = make_float2(0.f, 0.f);
#pragma unroll
                  for (int sa = 0; sa < 2; ++sa)
#pragma unroll
                    for (int sd = 0; sd < 2; ++sd)
                      cmac(k, TCV(sa, sb, sc, sd), Dad[(ia * 2 + sa) * MAXSP + id * 2 + sd]);
                  sadd(&K2[(ic * 2 + sc) * MAXSP + ib * 2 + sb], k);
                }
            }
          } else {
            // BRTMTZ: real parts, crossed exchange blocks
#pragma unroll
            for (int s = 0; s < 2; ++s) {
              float kv = 0.f;
#pragma unroll
              for (int t = 0; t < 2; ++t)
                kv = fmaf(TCV(s, t, t, s).x, Dcb[(ic * 2 + t) * MAXSP + ib * 2 + t].x, kv);
              atomicAdd(&Kl[(ia * 2 + s) * MAXSP + id * 2 + s].x, (double)kv);
            }
            if (dual) {
#pragma unroll
              for (int s = 0; s < 2; ++s) {
                float kv = 0.f;
#pragma unroll
                for (int t = 0; t < 2; ++t)
                  kv = fmaf(TCV(t, s, s, t).x, Dad[(ia * 2 + t) * MAXSP + id * 2 + t].x, kv);
                atomicAdd(&K2[(ic * 2 + s) * MAXSP + ib * 2 + s].x, (double)kv);
              }
            }
          }
#undef TCV
        }
        __syncthreads();
      }
    }
    if (abort) break;
    // flush; in a halved (LS|SL) list a quartet equal to its (dc|ba) image
    // counts 1/2 (the completion adds it again)
    const double wq = (q.dual == 2 && t2 == 1 && Q4.x == Q4.w && Q4.y == Q4.z) ? 0.5 : 1.0;
    for (int w = tid; w < 2 * nla * 2 * nld; w += NT) {
      int a = w / (2 * nld), d = w % (2 * nld);
      double2 v = Acc[a * MAXSP + d];
      if (v.x == 0.0 && v.y == 0.0) continue;
      int fa = A.fock[a >> 1][a & 1] + oa, fdd = Dd.fock[d >> 1][d & 1] + od;
      double *dst = q.BX + 2 * ((size_t)fa + (size_t)q.ldf * fdd);
      atomicAdd(dst, wq * v.x);
      atomicAdd(dst + 1, wq * v.y);
    }
    if (dual)
      for (int w = tid; w < 2 * nlc * 2 * nlb; w += NT) {
        int cc = w / (2 * nlb), b = w % (2 * nlb);
        double2 v = Acc[MAXSP * MAXSP + cc * MAXSP + b];
        if (v.x == 0.0 && v.y == 0.0) continue;
        int fcc = C.fock[cc >> 1][cc & 1] + oc, fbb = B.fock[b >> 1][b & 1] + ob;
        double *dst = q.BX + 2 * ((size_t)fcc + (size_t)q.ldf * fbb);
        atomicAdd(dst, wq * v.x);
        atomicAdd(dst + 1, wq * v.y);
      }
  }
  if (abort && tid == 0) atomicOr(&g_tc_status, 1);
  if (abort) {
    pipe_wait(pp, 0);
    pipe_wait(pp, 1);
  }
  fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                 :: "r"(tmem), "r"(q.tmem_cols));
}

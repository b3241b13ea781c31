/*
 * bertha_gpu.h - C ABI of the GB300 (sm_103a) Dirac-Coulomb Fock build.
 *
 * Drop-in for the reference's multi-centre Coulomb and Breit Fock builds:
 *   CALL EQSAVE   (bertha-scf.f:5287)  -> bertha_gpu_init
 *   CALL CLMFAST  (bertha-scf.f:5401)  -> bertha_gpu_clmfast
 *   CALL BRTFAST  (bertha-scf.f:5441)  -> bertha_gpu_brtfast
 * and, for a host SCF driver, the one-electron matrices:
 *   CALL OVRLP; CALL ONEEL (bertha-scf.f:5345-5346) -> bertha_gpu_oneel
 * The reference passes everything through COMMON blocks; here the same
 * arrays are passed explicitly, with their Fortran (column-major) layout and
 * leading dimensions, so a Fortran caller binds them with ISO_C_BINDING:
 *   /BSET/ BXYZ(3,MCT), NKAP(MCT), NFNC(0:MEL,MCT), BEXL(MBS,0:MEL,MCT)
 *   /DENS/ DENT(MDM,MDM)            COMPLEX*16
 *   /MTRX/ GDIR(MDM,MDM), GXCH(MDM,MDM), BXCH(MDM,MDM)   COMPLEX*16
 * Complex arrays are interleaved (re, im) doubles.  Every entry point
 * returns 0 on success or a BG_ERR_* code; none calls exit().
 * A context is used by one host thread at a time.
 */
#ifndef BERTHA_GPU_H
#define BERTHA_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define BG_OK 0
#define BG_ERR_ARG 1      /* invalid argument (reference: STOP in CARDIN) */
#define BG_ERR_CAPACITY 2 /* basis beyond the compiled limits */
#define BG_ERR_CUDA 3     /* CUDA runtime failure (message via last_error) */
#define BG_ERR_STATE 4    /* call on a context that failed earlier */

/* hmlt codes (CARDIN bertha-scf.f:224-233) */
#define BG_HMLT_NORL 0
#define BG_HMLT_BARE 1
#define BG_HMLT_DHFR 2
#define BG_HMLT_DHFP 3
#define BG_HMLT_DHFB 4
#define BG_HMLT_DHFQ 5

/* shape codes: ISYM of CLMFAST (bertha-scf.f:11569-11575) */
#define BG_SHAPE_GENERAL 0 /* 'PLANAR'/'NOSYMM': complex digestion (CLMMTG) */
#define BG_SHAPE_LINEAR 1  /* 'DIATOM'/'LINEAR': real digestion (CLMMTZ)   */
#define BG_SHAPE_ATOMIC 2  /* 'ATOMIC': real digestion (CLMMTZ)            */

/* init flags */
#define BG_FLAG_NO_RACAH1 1 /* include one-centre quartets (RACAH1=.FALSE.) */
#define BG_FLAG_GAUNT 2     /* Gaunt term only in the Breit build (GAUNT2) */

/* precision of the two-electron contraction */
#define BG_PREC_FP64 0 /* all FP64: the drop-in path */
#define BG_PREC_DF32 1 /* split precision: FP32 double-float contractions and
                          digestion products, FP64 Boys/R and J/K sums */
#define BG_PREC_AUTO 2 /* per angular class the fastest kernel within an
                          energy-error budget, chosen on the first build */
#define BG_PREC_TC32 3 /* tensor cores: both Hermite contractions as 3xTF32
                          tcgen05 GEMMs (FP32 accumulation), FP32 digestion
                          products, FP64 Boys/R and J/K sums */

/* compiled limits */
#define BG_MAX_L 3 /* highest orbital angular momentum of a basis shell */

typedef struct bg_ctx bg_ctx;

/* Build basis tables, the Fock layout of FOCKIND (bertha-scf.f:2582) and
 * all LL and SS E-coefficients on the device (EQSAVE, bertha-scf.f:32984).
 *   ncnt            NCNT
 *   bxyz[3*ncnt]    BXYZ, already translated/rotated by NUCGEOM
 *   nkap[ncnt]      NKAP = 2*LMAX+1 per centre
 *   nfnc            NFNC(0:MEL,MCT), column-major, leading dimension mel+1
 *   bexl            BEXL(MBS,0:MEL,MCT), leading dimensions mbs and mel+1
 *   hmlt, shape     BG_HMLT_*, BG_SHAPE_*
 *   flags           BG_FLAG_* */
int bertha_gpu_init(bg_ctx **ctx, int ncnt, const double *bxyz,
                    const int *nkap, const int *nfnc, int mel,
                    const double *bexl, int mbs, int hmlt, int shape,
                    int flags);

/* Select the contraction precision of later build calls (default FP64).
 * BG_PREC_DF32 carries every contraction operand as a pair of FP32 words
 * (about 48 significant bits) on the FP32 pipes.  No counterpart in the
 * reference, which is FP64 throughout. */
int bertha_gpu_set_precision(bg_ctx *ctx, int prec);

/* BG_PREC_AUTO is the autotuned mixed mode: the first build after the
 * quartet lists are made runs the FP64, the split-precision and the
 * tensor-core kernels on a sample of every angular class (l_a,l_b,l_c,l_d)
 * of every component class (classes under 2048 quartets take FP64), timing
 * each and comparing the sample's energy terms sum_ij Re D_ij G_ij (J and
 * K) with the FP64 kernel's.  Each class takes the faster of FP64 and the
 * split path (both FP64-accurate); classes then move to the tensor-core
 * kernel, largest time saved per estimated error first, while the summed
 * estimates (sample error x class size / sample size) stay within the
 * error budget (bertha_gpu_set_error_budget).  Later builds launch the
 * chosen kernel per run of classes.  Streamed lists and bertha_gpu_quartets
 * take the split kernel.  After a build, the quartets each kernel digests
 * and the number of runs (launches per build): */
int bertha_gpu_auto_stats(const bg_ctx *ctx, long long *nq_fp64, long long *nq_df32,
                          int *nruns);

/* The same with the tensor-core kernel: nq[0] FP64, nq[1] split, nq[2]
 * tensor-core quartets of the last tuned (or BG_PREC_TC32) build. */
int bertha_gpu_kernel_stats(const bg_ctx *ctx, long long nq[3], int *nruns);

/* Energy error (Eh) the BG_PREC_AUTO tuner may spend on tensor-core classes
 * per Coulomb build and, apart, per Breit build (default 1e-7 each, shared
 * equally by each build's component classes; 0 keeps every class
 * FP64-accurate).
 * Within a class, quartets are grouped by the decade of their Schwarz bound
 * Q_ab Q_cd, so that the small-magnitude part of a class can take the
 * tensor cores while its large part stays FP64.  Changing it retunes. */
int bertha_gpu_set_error_budget(bg_ctx *ctx, double eh);

/* The BG_PREC_AUTO tuner's record of the last tuning of the Coulomb
 * (breit = 0) or Breit (breit = 1) lists, one row per segment (angular
 * class and Schwarz-bound decade): info[4i..4i+3] = component class
 * (2*t1 + t2; Breit: 0 (LS|LS), 1 (LS|SL)), angular class
 * ((l_a*4 + l_b)*4 + l_c)*4 + l_d, quartets, chosen kernel (0 FP64,
 * 1 split, 2 tensor cores); vals[6i..6i+5] = sample time (ms) of the three
 * kernels (0 when not run) and their estimated energy errors (Eh).  At most
 * cap rows are written; *nrows gets the record's length.  After tuning the
 * library reorders its lists by chosen kernel, so the record is in tuning
 * order, not list order. */
int bertha_gpu_tuning_record(const bg_ctx *ctx, int breit, int cap, int *info, double *vals,
                             int *nrows);

/* Kernel use of the last Breit build (BG_PREC_AUTO or BG_PREC_TC32):
 * nq[0] FP64, nq[2] tensor-core quartets (nq[1] is 0: the Breit build has
 * no split-precision kernel). */
int bertha_gpu_breit_kernel_stats(const bg_ctx *ctx, long long nq[3], int *nruns);

/* Status of the tensor-core kernels since the last call (synchronises the
 * device): bit 0 set when an mbarrier wait gave up (the kernel skipped the
 * rest of its work, freed its tensor memory and returned), bit 1 when a
 * quartet's class needed more tensor memory than its launch allocated (the
 * quartet was skipped).  0 when every quartet was digested. */
int bertha_gpu_device_status(int *status);

/* Schwarz screening of the Fock build (SCHWARZ/CLMDIAG, bertha-scf.f:37889,
 * :38126; off by default there, SCHWRZ=.FALSE. :5257).  With threshold > 0,
 * shell quartets whose bound Q_ab Q_cd, Q = sqrt(max |(ab|ab)|) over labels,
 * m-signs and component, falls below it are skipped; 0 turns it off. */
int bertha_gpu_set_screening(bg_ctx *ctx, double threshold);

/* Quartet-list memory of the Coulomb build: a context keeps its lists on
 * the device while they hold at most cache_quartets quartets (0: 2^28);
 * larger lists are regenerated on the host every build and streamed
 * through pinned buffers of chunk_quartets quartets (0: 2^23), generation
 * overlapping the kernels of the previous chunk.  Cached lists make a build
 * capturable in a CUDA graph; streamed ones do not (they synchronise on
 * events).  No counterpart in the reference. */
int bertha_gpu_set_list_limits(bg_ctx *ctx, long long cache_quartets,
                               long long chunk_quartets);

/* Fock dimension NDIM and small-component offset NSKP (CARDIN :423-430). */
int bertha_gpu_dims(const bg_ctx *ctx, int *ndim, int *nskp);

/* Multi-centre Coulomb Fock build, replacing CALL CLMFAST
 * (bertha-scf.f:11489-12266).  Host arrays:
 *   dent[ldd*ndim]  total density DENT (complex, column-major)
 *   ilev            integral inclusion stage ILEV (1..4)
 *   gdir, gxch      [ldf*ndim] outputs, overwritten (CLMFAST zeroes them)
 * Semantics follow CLMFAST with CLMMTG (shape GENERAL) or CLMMTZ (LINEAR,
 * ATOMIC) digestion; one-centre quartets are skipped unless
 * BG_FLAG_NO_RACAH1 was given.  Like CLMFAST with INTSYM (its default), the
 * build evaluates a symmetry-reduced quartet set and completes GDIR and GXCH
 * as Hermitian matrices (:12164-12205), which assumes a Hermitian DENT (as
 * DENSTY makes it). */
int bertha_gpu_clmfast(bg_ctx *ctx, const double *dent, int ldd, int ilev,
                       double *gdir, double *gxch, int ldf);

/* Same build on device-resident arrays, stream-ordered on `stream`
 * (a cudaStream_t, or NULL for the default stream). */
int bertha_gpu_clmfast_device(bg_ctx *ctx, const double *d_dent, int ldd,
                              int ilev, double *d_gdir, double *d_gxch,
                              int ldf, void *stream);

/* Closed-shell multi-centre Breit exchange matrix, replacing CALL BRTFAST
 * (bertha-scf.f:17060-17670; BIIFAST :18337, BRTMTG :19815, BRTMTZ :19172).
 * Precision: FP64 by default; BG_PREC_TC32 runs every class on the tensor
 * cores (k_breit_tc, 3xTF32), BG_PREC_AUTO tunes per class and bound decade
 * within the error budget; BG_PREC_DF32 leaves the Breit build FP64.
 *   dent[ldd*ndim]  total density DENT
 *   ilev            ILEV: multi-centre quartets from stage 3 on (:17230-17231)
 *   bxch[ldf*ndim]  output BXCH, overwritten
 * Full Breit interaction -1/2 [a1.a2/r12 + (a1.r12)(a2.r12)/r12^3], or the
 * Gaunt term -a1.a2/r12 alone when the context was made with BG_FLAG_GAUNT.
 * BDIR is zero for closed shells and not produced.  The SL block is the
 * conjugate transpose of the LS block, as BRTFAST completes it.  Needs a
 * four-component Hamiltonian (BG_ERR_ARG for NORL and BARE); the reference
 * calls it for DHFB and DHFQ.  The first call generates the sigma-coupled
 * LS/SL E-coefficients (EILS/EISL of EQSAVE).  The (LS|SL) quartets that
 * feed the LL and SS blocks are halved by (dc|ba) = (ab|cd)* and those
 * blocks completed as Hermitian matrices, which assumes a Hermitian DENT. */
int bertha_gpu_brtfast(bg_ctx *ctx, const double *dent, int ldd, int ilev,
                       double *bxch, int ldf);

/* Same build on device-resident arrays, stream-ordered on `stream`. */
int bertha_gpu_brtfast_device(bg_ctx *ctx, const double *d_dent, int ldd,
                              int ilev, double *d_bxch, int ldf, void *stream);

/* One-electron matrices, replacing CALL OVRLP and CALL ONEEL
 * (bertha-scf.f:6683, 6996-7990):
 *   znuc[ncnt]   nuclear charges ZNUC
 *   xi[ncnt]     Gaussian nuclear exponents XNUC(IZ,0) = 1.5/RNUC^2 of
 *                NUCCOUL (:1183-1210), 0 for a point nucleus
 *   ovlp, hnuc, hkin [ldf*ndim] outputs, overwritten: OVLP (LL and SS
 *                blocks), HNUC (nuclear attraction; SS block minus
 *                2 c^2 S_SS), HKIN (c sigma.p couplings between L and S, or
 *                the non-relativistic kinetic matrix for NORL). */
int bertha_gpu_oneel(bg_ctx *ctx, const double *znuc, const double *xi,
                     double *ovlp, double *hnuc, double *hkin, int ldf);

/* Same on device-resident outputs (znuc, xi stay host arrays). */
int bertha_gpu_oneel_device(bg_ctx *ctx, const double *znuc, const double *xi,
                            double *d_ovlp, double *d_hnuc, double *d_hkin,
                            int ldf, void *stream);

/* Fock-build digestion over an explicit list of ordered shell quartets
 * (device array, 4 ints each: shell a, b, c, d as numbered by
 * bertha_gpu_shells, each in [0, nshell); the device list is not checked,
 * so an index outside that range reads past the shell tables) with
 * component classes t1 (ab) and t2 (cd), 0 = LL and
 * 1 = SS.  Adds, without zeroing, J(a,b) += (ab|cd) D(c,d) and
 * K(a,d) += (ab|cd) D(c,b) over every spinor label and m-sign of each
 * quartet: batch types 1 and 5 of CLMMTG/CLMMTZ (bertha-scf.f:13841). */
int bertha_gpu_quartets(bg_ctx *ctx, const int *d_quartets, long long nq,
                        int t1, int t2, const double *d_dent, int ldd,
                        double *d_gdir, double *d_gxch, int ldf, void *stream);

/* bertha_gpu_quartets over a list the caller has grouped by angular class:
 * nseg segments, entries seg[i]..seg[i+1]-1 (host array of nseg+1 offsets
 * into d_quartets) all of class lclass[4i..4i+3] = (l_a, l_b, l_c, l_d)
 * (host array).  Under BG_PREC_TC32 each run of classes gets a launch sized
 * for its tensor-memory need (more CTAs per SM for small classes); other
 * precisions digest the whole range in one launch as bertha_gpu_quartets
 * does.  A quartet whose class needs more tensor memory than its segment's
 * class is skipped and flagged (bertha_gpu_device_status). */
int bertha_gpu_quartets_segments(bg_ctx *ctx, const int *d_quartets, int nseg,
                                 const long long *seg, const int *lclass, int t1, int t2,
                                 const double *d_dent, int ldd, double *d_gdir,
                                 double *d_gxch, int ldf, void *stream);

/* Largest NDIM bertha_gpu_quartets_noalloc accepts. */
#define BG_NOALLOC_MAX_NDIM 1024

/* Same digestion as bertha_gpu_quartets in split precision (BG_PREC_DF32),
 * for callers that cannot allocate device memory: code running inside an
 * application whose memory pool already owns the GPU's memory, or issuing
 * work where a cudaMalloc would synchronise the device.  It allocates
 * nothing: its only scratch, the double-float copy of the density, is a
 * static device array of BG_NOALLOC_MAX_NDIM^2 x 16 bytes (16 MiB) that every
 * GPU loading the library holds until exit.  Contexts with NDIM above
 * BG_NOALLOC_MAX_NDIM get BG_ERR_CAPACITY.  The first call on a device looks
 * up the array's device address (cudaGetSymbolAddress), so make that first
 * call before any stream capture.  All calls share the array: calls that
 * overlap on the GPU race on it.  The context itself comes from
 * bertha_gpu_init as usual.  No counterpart in the reference. */
int bertha_gpu_quartets_noalloc(bg_ctx *ctx, const int *d_quartets,
                                long long nq, int t1, int t2,
                                const double *d_dent, int ldd, double *d_gdir,
                                double *d_gxch, int ldf, void *stream);

/* Batched Fock builds of independent instances (atoms, ions, molecules of
 * different basis sizes), one kernel launch per component class for all
 * of them.  The reference runs such instances as separate bertha-scf
 * processes; this replaces CALL CLMFAST (bertha-scf.f:5401) of each of them
 * by one stream-ordered call.  No counterpart in the reference. */
typedef struct bg_batch bg_batch;

/* Make a batch from n contexts (bertha_gpu_init).  The instances must share
 * hmlt, shape and the RACAH1 flag; each keeps its own Schwarz threshold
 * (bertha_gpu_set_screening before this call) and quartet rules.  The batch
 * copies what it needs: the contexts may be freed afterwards.  Placement of
 * the matrices in the batch's device arrays: element (i, j) of instance k's
 * density and outputs is complex element moff[k] + i + ld[k]*j; moff = NULL
 * packs the instances one after another with ld = NDIM (ld = NULL: NDIM).
 * The precision is taken from ctxs[0] (bertha_gpu_set_precision). */
int bertha_gpu_batch_create(bg_batch **b, int n, bg_ctx *const *ctxs,
                            const long long *moff, const int *ld);

/* Contraction precision of the batch's later builds (BG_PREC_*; with
 * BG_PREC_AUTO the batch's merged lists are tuned per angular class on the
 * first build, as for a context). */
int bertha_gpu_batch_set_precision(bg_batch *b, int prec);

/* bertha_gpu_auto_stats, bertha_gpu_kernel_stats and
 * bertha_gpu_set_error_budget of a batch (the budget covers the whole
 * batch's build). */
int bertha_gpu_batch_auto_stats(const bg_batch *b, long long *nq_fp64, long long *nq_df32,
                                int *nruns);
int bertha_gpu_batch_kernel_stats(const bg_batch *b, long long nq[3], int *nruns);
int bertha_gpu_batch_set_error_budget(bg_batch *b, double eh);

/* CLMFAST of every instance at stage ilev on device arrays in the batch's
 * placement: d_dent holds all densities; d_gdir, d_gxch get all GDIR and
 * GXCH, each instance's NDIM x NDIM block overwritten (other elements are
 * left alone).  Like bertha_gpu_clmfast, each instance's density must be
 * Hermitian (the build is symmetry-reduced and completed).  The first call
 * at a stage builds the quartet lists (host work and allocation; under
 * BG_PREC_AUTO it also tunes the kernel choice); later calls at that stage
 * only launch kernels on `stream` and can be captured in a CUDA graph. */
int bertha_gpu_batch_clmfast_device(bg_batch *b, const double *d_dent, int ilev,
                                    double *d_gdir, double *d_gxch, void *stream);

/* Shell quartets in the batch's lists at the last stage built. */
long long bertha_gpu_batch_quartets(const bg_batch *b);

/* Kernel launches issued by the last batched build call. */
long long bertha_gpu_batch_launches(const bg_batch *b);

/* Message of the last error on this batch (or of bertha_gpu_batch_create
 * when b is NULL). */
const char *bertha_gpu_batch_last_error(const bg_batch *b);

void bertha_gpu_batch_free(bg_batch *b);

/* Number of primitive shells and, per shell (centre, l, index in the
 * exponent list), in the order centre, l, exponent. */
int bertha_gpu_shells(const bg_ctx *ctx, int *nshell, int *cnt, int *l,
                      int *ibas);

/* LRGE Fock offsets (FOCKIND): lrge[(cnt*(2*BG_MAX_L+2) + ka)*28 + m],
 * ka = KA (1-based), m = 2|m_j|-1 + (m_j > 0). */
int bertha_gpu_layout(const bg_ctx *ctx, int *lrge);

/* Kernel launches issued by the last build call. */
long long bertha_gpu_launches(const bg_ctx *ctx);

/* Message of the last error on this context (or on init when ctx is NULL). */
const char *bertha_gpu_last_error(const bg_ctx *ctx);

void bertha_gpu_free(bg_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif

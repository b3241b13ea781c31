"""GPU Fock build against the oracle, through the C ABI.

Tolerance: both sides are FP64; they differ only in summation order (the
GPU accumulates with atomics), so the bound is 1e-11 relative to the
largest matrix element.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import berthagpu  # noqa: E402
from berthagpu import deck  # noqa: E402
from oracle import oracle as orc  # noqa: E402

TOL = 1e-11


def _small(isym=None, hmlt="DHFR", lmax=1):
    cent = [((0.0, 0.0, 0.0), {0: [0.3, 2.5], 1: [0.7]}),
            ((0.3, -0.8, 1.3), {0: [0.45], 1: [1.1]}),
            ((-1.0, 0.5, 0.4), {0: [0.9, 0.2]})]
    if lmax >= 2:
        cent[0][1][2] = [0.8]
    if lmax >= 3:
        cent[1][1][3] = [0.6]
    return deck.make_basis(cent, hmlt=hmlt, isym=isym)


def _cmp(b, dent, ilev, racah1=True):
    fb = berthagpu.FockBuilder(b, racah1=racah1)
    gd, gx = fb.clmfast(dent, ilev)
    fb.close()
    rd, rx = orc.clmfast(b, dent, ilev, racah1=racah1)
    scale = max(np.abs(rd).max(), np.abs(rx).max(), 1e-300)
    assert np.abs(gd - rd).max() <= TOL * scale
    assert np.abs(gx - rx).max() <= TOL * scale
    return rd, rx


@pytest.mark.parametrize("ilev", [1, 2, 3])
def test_small_general(ilev):
    b = _small()
    _cmp(b, deck.density(b, seed=ilev), ilev)


@pytest.mark.parametrize("lmax", [2, 3])
def test_small_high_l(lmax):
    b = _small(lmax=lmax)
    _cmp(b, deck.density(b, seed=11), 3)


def test_linear_real_digestion():
    """DIATOM/LINEAR: CLMMTZ semantics (real parts, m-selection)."""
    b = deck.make_basis([((0, 0, 0), {0: [0.4, 1.9], 1: [0.8], 2: [1.2]}),
                         ((0, 0, 2.1), {0: [0.6], 1: [0.5]})], hmlt="DHFR")
    assert b.isym == 1
    _cmp(b, deck.density(b, seed=5, real=True), 3)


def test_norl():
    b = _small(hmlt="NORL")
    _cmp(b, deck.density(b, seed=3), 1)


def test_one_centre_by_md():
    """RACAH1 off: one-centre quartets through the MD path with the atomic
    selection rules of CLMFAST (bertha-scf.f:11753-11939)."""
    b = _small()
    _cmp(b, deck.density(b, seed=9), 3, racah1=False)


def test_h2o_stage1():
    b = deck.h2o_basis()
    _cmp(b, deck.density(b, seed=1), 1)


def test_bad_arguments():
    b = _small()
    fb = berthagpu.FockBuilder(b)
    with pytest.raises(berthagpu.BerthaGPUError):
        fb.clmfast(np.zeros((3, 3), complex), 1)
    with pytest.raises(berthagpu.BerthaGPUError):
        fb.clmfast(deck.density(b), 7)
    fb.close()


def test_capacity_error():
    """An l=4 shell is beyond the compiled limit: BG_ERR_CAPACITY, not a crash."""
    b = _small()
    lmax = b.lmax.copy()
    lmax[0] = 4
    nfn = np.zeros((b.ncnt, 5), np.int32)
    nfn[:, :4] = b.nfn
    nfn[0, 4] = 1
    ex = np.zeros((b.ncnt, 5, b.ex.shape[2]))
    ex[:, :4] = b.ex
    ex[0, 4, 0] = 1.0
    bad = deck.Basis(xyz=b.xyz, lmax=lmax, nfn=nfn, ex=ex, hmlt=b.hmlt, isym=b.isym)
    with pytest.raises(berthagpu.BerthaGPUError) as ei:
        berthagpu.FockBuilder(bad)
    assert ei.value.code == 2


# Split precision: FP32 double-float contractions.  Tolerance 1e-10 of the
# largest element (about 2^-44 per operation, with cancellation headroom).
DF_TOL = 1e-10


def _cmp_df(b, dent, ilev):
    fb = berthagpu.FockBuilder(b)
    fb.set_precision("df32")
    gd, gx = fb.clmfast(dent, ilev)
    fb.close()
    rd, rx = orc.clmfast(b, dent, ilev)
    scale = max(np.abs(rd).max(), np.abs(rx).max(), 1e-300)
    assert np.abs(gd - rd).max() <= DF_TOL * scale
    assert np.abs(gx - rx).max() <= DF_TOL * scale


@pytest.mark.parametrize("lmax", [1, 3])
def test_df32_general(lmax):
    b = _small(lmax=lmax)
    _cmp_df(b, deck.density(b, seed=21), 3)


def test_df32_linear():
    b = deck.make_basis([((0, 0, 0), {0: [0.4, 1.9], 1: [0.8], 2: [1.2]}),
                         ((0, 0, 2.1), {0: [0.6], 1: [0.5]})], hmlt="DHFR")
    _cmp_df(b, deck.density(b, seed=5, real=True), 3)


def test_df32_extreme_exponents():
    """Exponent ratios up to 1e7 exercise the power-of-two scaling."""
    b = deck.make_basis([((0, 0, 0), {0: [0.05, 2.0e5], 1: [3.0e4], 2: [0.3]}),
                         ((0.4, 1.1, -0.7), {0: [1.0e6, 0.08], 1: [0.1]}),
                         ((1.5, -0.3, 0.9), {0: [0.5], 3: [40.0]})], hmlt="DHFR")
    _cmp_df(b, deck.density(b, seed=8), 3)


def test_schwarz_screening():
    """Shell-pair Schwarz screening: at 1e-12 the Fock matrices stay within
    1e-9 (absolute) of the unscreened oracle; a huge threshold removes every
    quartet (so the screen is really applied)."""
    b = deck.make_basis([((0, 0, 0), {0: [0.1, 50.0, 5.0e4], 1: [0.3, 2.0e3]}),
                         ((0, 0, 6.0), {0: [0.2, 8.0e4], 1: [1.0e3]}),
                         ((5.0, 1.0, 2.0), {0: [0.15, 3.0e4]})], hmlt="DHFR")
    dent = deck.density(b, seed=13)
    rd, rx = orc.clmfast(b, dent, 3)
    fb = berthagpu.FockBuilder(b)
    fb.set_screening(1e-12)
    gd, gx = fb.clmfast(dent, 3)
    assert np.abs(gd - rd).max() <= 1e-9 and np.abs(gx - rx).max() <= 1e-9
    fb.set_screening(1e3)
    gd, gx = fb.clmfast(dent, 3)
    assert np.abs(gd).max() == 0.0 and np.abs(gx).max() == 0.0
    fb.set_screening(0.0)
    gd, gx = fb.clmfast(dent, 3)
    scale = max(np.abs(rd).max(), np.abs(rx).max())
    assert np.abs(gd - rd).max() <= TOL * scale
    fb.close()


@pytest.mark.parametrize("prec", ["fp64", "df32", "auto"])
def test_streamed_quartet_lists(prec):
    """Lists above the cache limit are regenerated and streamed in chunks:
    tiny limits force several chunks per class on a small basis (the
    autotuned mode takes the split kernel for streamed lists)."""
    b = _small(lmax=2)
    d = deck.density(b, seed=41)
    fb = berthagpu.FockBuilder(b)
    fb.set_precision(prec)
    fb.set_screening(1e-12)
    fb.set_list_limits(1000, 777)
    gd, gx = fb.clmfast(d, 3)
    gd2, gx2 = fb.clmfast(d, 3)
    fb.close()
    rd, rx = orc.clmfast(b, d, 3)
    scale = max(np.abs(rd).max(), np.abs(rx).max())
    tol = (TOL if prec == "fp64" else DF_TOL) * scale + 1e-9
    for g, r in ((gd, rd), (gx, rx), (gd2, rd), (gx2, rx)):
        assert np.abs(g - r).max() <= tol


def test_h2o_stage3_fp64():
    """The H2O configuration at ILEV 3 (all four component classes), FP64,
    against the oracle."""
    b = deck.h2o_basis()
    _cmp(b, deck.density(b, seed=2), 3)


def _explicit(fb, q, cls, dent):
    import torch
    n = fb.ndim
    D = torch.from_numpy(np.ascontiguousarray(dent.T).view(np.float64).reshape(n, 2 * n)).cuda()
    GD = torch.zeros(n, 2 * n, dtype=torch.float64, device="cuda")
    GX = torch.zeros_like(GD)
    dq = torch.from_numpy(np.ascontiguousarray(q, dtype=np.int32)).cuda()
    fb.quartets(dq.data_ptr(), q.shape[0], cls[0], cls[1], D.data_ptr(), GD.data_ptr(),
                GX.data_ptr(), n, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return (GD.cpu().numpy().view(np.complex128).reshape(n, n).T,
            GX.cpu().numpy().view(np.complex128).reshape(n, n).T)


def _oracle_explicit(b, q, cls, dent):
    n = b.ndim
    rd = np.zeros((n, n), complex, order="F")
    rx = np.zeros((n, n), complex, order="F")
    O = orc.QuartetOracle(b)
    O.prepare(q, *cls)
    O.digest(q, *cls, dent, rd, rx, nthreads=16)
    O.close()
    return rd, rx


def _class_sample(b, per_class, seed):
    """Seeded quartets of every angular class (l_a,l_b,l_c,l_d) of a basis,
    shells drawn at random among those of each l (every centre)."""
    rng = np.random.default_rng(seed)
    sh = b.shells()
    byl = {}
    for s, (c, l, i, _) in enumerate(sh):
        byl.setdefault(l, []).append(s)
    out = []
    ls = sorted(byl)
    for la in ls:
        for lb in ls:
            for lc in ls:
                for ld in ls:
                    for _ in range(per_class):
                        out.append([rng.choice(byl[x]) for x in (la, lb, lc, ld)])
    return np.array(out, dtype=np.int32)


@pytest.mark.parametrize("prec", ["fp64", "df32", "auto", "tc32"])
def test_tlf_full_basis_class_sample(prec):
    """The full TlF basis (Tl exponents up to 0.02 * 2.2^27, about 3.6e7) on
    a seeded sample of every angular class of every component class, through
    explicit lists against the oracle.  The shape is taken as GENERAL so that
    both sides use the complex digestion (the oracle's explicit-list path has
    no real-digestion mode); the integrals are those of the linear molecule."""
    b0 = deck.tlf_basis()
    b = deck.Basis(xyz=b0.xyz, lmax=b0.lmax, nfn=b0.nfn, ex=b0.ex, hmlt=deck.HMLT["DHFR"],
                   isym=0, name="TlF")
    q = _class_sample(b, 2, seed=17)
    dent = deck.density(b, seed=4)
    fb = berthagpu.FockBuilder(b)
    fb.set_precision(prec)
    tol = {"fp64": TOL, "df32": DF_TOL, "auto": DF_TOL, "tc32": 2e-5}[prec]
    for cls in ((0, 0), (0, 1), (1, 0), (1, 1)):
        gd, gx = _explicit(fb, q, cls, dent)
        rd, rx = _oracle_explicit(b, q, cls, dent)
        scale = max(np.abs(rd).max(), np.abs(rx).max())
        assert np.abs(gd - rd).max() <= tol * scale, cls
        assert np.abs(gx - rx).max() <= tol * scale, cls
    fb.close()


def test_microbench_quartets_vs_oracle():
    """4096 quartets of the ERI microbenchmark's distribution (l <= 3,
    exponents 0.05..1e6, 20 % overlapping pairs) against the oracle, FP64
    and split precision."""
    from berthagpu import workloads
    b = workloads.microbench_pool(seed=5, ncentres=12)
    quarts = workloads.microbench_quartets(b, 4096, seed=5)
    dent = deck.density(b, seed=5)
    for prec, tol in (("fp64", TOL), ("df32", DF_TOL)):
        fb = berthagpu.FockBuilder(b)
        fb.set_precision(prec)
        for cls, q in quarts.items():
            gd, gx = _explicit(fb, q, cls, dent)
            rd, rx = _oracle_explicit(b, q, cls, dent)
            scale = max(np.abs(rd).max(), np.abs(rx).max())
            assert np.abs(gd - rd).max() <= tol * scale, (prec, cls)
            assert np.abs(gx - rx).max() <= tol * scale, (prec, cls)
        fb.close()

"""Host-side workload definitions, on the CPU: the closed-shell atom
batch's basis sizes, and the halved (LS|SL) Breit list's coverage of every
ordered quartet through the (dc|ba) = (ab|cd)* relation."""
import numpy as np

from berthagpu import deck, workloads


def test_atom_basis_sizes():
    # n_s = 8 + Z/4, n_p = 6 + Z/5, n_d = Z/12, n_f = Z/24 (integer division)
    he, rn = deck.atom_basis(2), deck.atom_basis(86)
    assert he.ndim == 104 and rn.ndim == 616
    assert list(rn.nfn[0]) == [29, 23, 7, 3]
    assert rn.isym == deck.SHAPE["ATOMIC"]
    assert abs(rn.ex[0, 0, 0] - 0.03) < 1e-15 and abs(rn.ex[0, 0, 1] / rn.ex[0, 0, 0] - 2.4) < 1e-12


def test_batched_atoms_draw():
    a = deck.batched_atoms(96, seed=2024)
    b = deck.batched_atoms(96, seed=2024)
    assert len(a) == 96
    assert [x.znuc for x in a] == [x.znuc for x in b]
    assert {int(x.znuc[0]) for x in a} <= set(deck.CLOSED_SHELL_ATOMS)
    assert min(x.ndim for x in a) >= 104 and max(x.ndim for x in a) <= 616
    light = deck.batched_atoms(16, seed=1, zset=[2, 4])
    assert {int(x.znuc[0]) for x in light} <= {2, 4}


def test_breit_ls_sl_halving_covers_every_quartet():
    b = deck.make_basis([((0, 0, 0), {0: [0.4, 2.0], 1: [0.9]}),
                         ((0.0, 0.6, 1.1), {0: [0.7], 1: [1.5]})], hmlt="DHFB")
    q_lsls, q_lssl = workloads.breit_quartets(b, racah1=False)
    ns = len(b.shells())
    listed = {tuple(x) for x in q_lssl}
    # the full (LS|SL) class under the same centre and parity rules
    a, bb, c, d = (x.ravel() for x in np.meshgrid(*(np.arange(ns),) * 4, indexing="ij"))
    l = np.array([s[1] for s in b.shells()])
    keep = ((l[a] + l[bb]) & 1) == ((l[c] + l[d]) & 1)
    cnt = np.array([s[0] for s in b.shells()])
    multi = ~((cnt[a] == cnt[bb]) & (cnt[a] == cnt[c]) & (cnt[a] == cnt[d]))
    keep |= multi
    allq = {(int(w), int(x), int(y), int(z)) for w, x, y, z, k in zip(a, bb, c, d, keep) if k}
    # every quartet is listed or its (dc|ba) image is, never both unless
    # they are the same quartet
    for (w, x, y, z) in allq:
        img = (z, y, x, w)
        assert ((w, x, y, z) in listed) != (img in listed) or img == (w, x, y, z)
    assert listed <= allq
    assert len(q_lsls) > 0


def test_quartet_oracle_layout_matches_basis():
    """The oracle's explicit-list context uses the basis's own Fock layout:
    a four-component basis has its small component at NSKP = NDIM/2 (the
    layout the library and the oracle's CLMFAST use), a NORL basis none."""
    from oracle import oracle as orc
    b = deck.make_basis([((0, 0, 0), {0: [0.4, 2.0], 1: [0.9]}),
                         ((0.0, 0.6, 1.1), {0: [0.7]})], hmlt="DHFR")
    O = orc.QuartetOracle(b)
    assert O.ndim == b.ndim and O.nskp == b.ndim // 2
    O.close()
    bn = deck.make_basis([((0, 0, 0), {0: [0.4, 2.0], 1: [0.9]})], hmlt="NORL")
    O = orc.QuartetOracle(bn)
    assert O.ndim == bn.ndim and O.nskp == 0
    O.close()


def test_group_by_class_segments():
    b = workloads.microbench_pool(seed=3, ncentres=4)
    q = workloads.microbench_quartets(b, 2000, seed=3)[(0, 1)]
    qq, seg, lcl = workloads.group_by_class(b, q)
    l = np.array([s[1] for s in b.shells()])
    assert sorted(map(tuple, qq)) == sorted(map(tuple, q))
    assert seg[0] == 0 and seg[-1] == len(q)
    for i in range(len(seg) - 1):
        part = qq[seg[i]:seg[i + 1]]
        assert (np.stack([l[part[:, j]] for j in range(4)], 1) == lcl[i]).all()

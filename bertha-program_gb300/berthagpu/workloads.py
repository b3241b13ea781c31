"""Seeded synthetic workloads.

ERI microbenchmark: random shell quartets over a pool of primitive shells.
Angular momenta l_a..l_d are uniform on {0,1,2,3}; exponents are
log-uniform on [0.05, 1e6]; centres are uniform in a 10-bohr cube, and the
second shell of a pair sits on the first one's centre in 20% of pairs.  The
quartets are split evenly over the four component classes LL|LL, LL|SS,
SS|LL and SS|SS (the SS partners carry l+1 through kinetic balance).
"""
import numpy as np

from .deck import make_basis

CLASSES = ((0, 0), (0, 1), (1, 0), (1, 1))


def microbench_pool(seed=2024, ncentres=32, nexp=2, lmax=3, cube=10.0,
                    emin=0.05, emax=1.0e6):
    rng = np.random.default_rng(seed)
    cents = []
    for _ in range(ncentres):
        pos = rng.uniform(0.0, cube, 3)
        d = {l: list(np.exp(rng.uniform(np.log(emin), np.log(emax), nexp)))
             for l in range(lmax + 1)}
        cents.append((pos, d))
    return make_basis(cents, hmlt="DHFR", isym=0, name="eri-pool")


def shell_index(basis):
    """shell id of (centre, l, i) in the library's order"""
    idx = {}
    for s, (c, l, i, _) in enumerate(basis.shells()):
        idx[(c, l, i)] = s
    return idx


def microbench_quartets(basis, nquart, seed=2024, overlap=0.2):
    """Returns {(t1,t2): int32 array [n,4]} with nquart quartets in total."""
    rng = np.random.default_rng(seed + 1)
    idx = shell_index(basis)
    nc = basis.ncnt
    lmax = int(basis.lmax.min())
    nexp = int(basis.nfn[:, : lmax + 1].min())
    out = {}
    per = nquart // len(CLASSES)
    for k, cls in enumerate(CLASSES):
        n = per if k < len(CLASSES) - 1 else nquart - per * (len(CLASSES) - 1)
        ls = rng.integers(0, lmax + 1, size=(n, 4))
        ca = rng.integers(0, nc, size=n)
        cc = rng.integers(0, nc, size=n)
        cb = np.where(rng.random(n) < overlap, ca, (ca + rng.integers(1, nc, size=n)) % nc)
        cd = np.where(rng.random(n) < overlap, cc, (cc + rng.integers(1, nc, size=n)) % nc)
        cen = np.stack([ca, cb, cc, cd], 1)
        q = np.empty((n, 4), np.int32)
        for j in range(4):
            ii = rng.integers(0, nexp, size=n)
            q[:, j] = [idx[(int(c), int(l), int(i))] for c, l, i in zip(cen[:, j], ls[:, j], ii)]
        out[cls] = q
    return out


def quartet_flops(basis, quart, t1, t2):
    """Algorithmic FP64 flops of a quartet list: Boys+R recursion
    (6 per R entry up to the class order), first contraction
    2*(4P_ab)*N_ab*N_cd and second contraction 2*(4P_ab)*(4P_cd)*N_cd."""
    sh = basis.shells()
    l = np.array([s[1] for s in sh])
    la, lb, lc, ld = (l[quart[:, j]] for j in range(4))

    def nt(L):
        return (L + 1) * (L + 2) * (L + 3) // 6

    degab = la + lb + 2 * t1
    degcd = lc + ld + 2 * t2
    lam = degab + degcd
    pab = (2 * la + 1) * (2 * lb + 1)
    pcd = (2 * lc + 1) * (2 * ld + 1)
    fr = 6 * np.array([sum(nt(k) for k in range(int(L) + 1)) for L in lam])
    f1 = 2 * (4 * pab) * nt(degab) * nt(degcd)
    f2 = 2 * (4 * pab) * (4 * pcd) * nt(degcd)
    return float(np.sum(fr + f1 + f2))


def contraction_flops(basis, quart, t1, t2):
    """Dense Hermite-contraction flops of a quartet list (the tensor-core
    work): first contraction 2*(4P_ab)*N_ab*N_cd and second 2*(4P_ab)*(4P_cd)*N_cd
    per quartet (the R recursion excluded)."""
    sh = basis.shells()
    l = np.array([s[1] for s in sh])
    la, lb, lc, ld = (l[quart[:, j]] for j in range(4))

    def nt(L):
        return (L + 1) * (L + 2) * (L + 3) // 6

    degab = la + lb + 2 * t1
    degcd = lc + ld + 2 * t2
    pab = (2 * la + 1) * (2 * lb + 1)
    pcd = (2 * lc + 1) * (2 * ld + 1)
    f1 = 2 * (4 * pab) * nt(degab) * nt(degcd)
    f2 = 2 * (4 * pab) * (4 * pcd) * nt(degcd)
    return float(np.sum(f1 + f2))


def breit_quartets(basis, ilev=3, racah1=True):
    """Shell quartets of the Breit build as the library lists them
    (BRTFAST centre and stage rules): (LS|LS) with pair index ab >= cd and
    (LS|SL) with (ab, cd) >= (dc, ba) in pair-index order (one of each
    quartet and its conjugate image (dc|ba)); returns the two int32 [n, 4]
    arrays."""
    sh = basis.shells()
    cnt = np.array([s[0] for s in sh])
    l = np.array([s[1] for s in sh])
    ns = len(sh)
    a, b, c, d = (x.ravel() for x in np.meshgrid(*(np.arange(ns),) * 4, indexing="ij"))
    cen = np.sort(np.stack([cnt[a], cnt[b], cnt[c], cnt[d]], 1), 1)
    mcnt = 1 + (np.diff(cen, axis=1) != 0).sum(1)
    keep = np.ones(a.shape, bool)
    if racah1:
        keep &= mcnt != 1
    if ilev < 3:
        keep &= mcnt == 1
    keep &= (mcnt != 1) | (((l[a] + l[b]) & 1) == ((l[c] + l[d]) & 1))
    pab, pcd = a * ns + b, c * ns + d
    pdc, pba = d * ns + c, b * ns + a
    q = np.stack([a, b, c, d], 1).astype(np.int32)
    half = (pab > pdc) | ((pab == pdc) & (pcd >= pba))
    return q[keep & (pab >= pcd)], q[keep & half]


def breit_flops(basis, quart, gaunt=False):
    """Algorithmic FP64 flops of a Breit quartet list: R to order
    Lambda_ab+Lambda_cd+2 (6 per entry), first contraction over three
    Cartesian components of each electron 2*(4P_ab)*N_ab*N_cd*9 (3 for Gaunt)
    and second contraction 2*(4P_ab)*(4P_cd)*N_cd*3, N of degree la+lb+1."""
    sh = basis.shells()
    l = np.array([s[1] for s in sh])
    la, lb, lc, ld = (l[quart[:, j]] for j in range(4))

    def nt(L):
        return (L + 1) * (L + 2) * (L + 3) // 6

    degab, degcd = la + lb + 1, lc + ld + 1
    lam = degab + degcd + (0 if gaunt else 2)
    pab = (2 * la + 1) * (2 * lb + 1)
    pcd = (2 * lc + 1) * (2 * ld + 1)
    cum = np.cumsum([nt(k) for k in range(40)])
    fr = 6 * cum[lam]
    f1 = 2 * (4 * pab) * nt(degab) * nt(degcd) * (3 if gaunt else 9)
    f2 = 2 * (4 * pab) * (4 * pcd) * nt(degcd) * 3
    return float(np.sum(fr + f1 + f2))


def group_by_class(basis, quart):
    """A quartet list reordered by angular class (l_a,l_b,l_c,l_d), highest
    first (the order in which CLMFAST visits its L blocks), with its segment
    table: returns (quartets, seg, lclass) where entries seg[i]..seg[i+1]-1
    have angular momenta lclass[i] (the arguments of
    bertha_gpu_quartets_segments)."""
    l = np.array([s[1] for s in basis.shells()])
    ls = np.stack([l[quart[:, j]] for j in range(4)], 1)
    key = ((ls[:, 0] * 4 + ls[:, 1]) * 4 + ls[:, 2]) * 4 + ls[:, 3]
    order = np.argsort(-key, kind="stable")
    q = np.ascontiguousarray(quart[order])
    ks = key[order]
    starts = np.flatnonzero(np.r_[True, ks[1:] != ks[:-1]]) if len(ks) else np.zeros(0, int)
    seg = np.r_[starts, len(ks)].astype(np.int64)
    lclass = ls[order][starts].astype(np.int32)
    return q, seg, lclass

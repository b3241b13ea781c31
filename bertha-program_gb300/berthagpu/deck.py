"""Basis description and input-deck reader (the CARDIN input format).

``Basis`` holds the arrays of the reference's COMMON /BSET/ in the layout
the C ABI takes: centre coordinates BXYZ, LMAX per centre (NKAP = 2*LMAX+1),
NFNC(0:MEL,MCT) and BEXL(MBS,0:MEL,MCT) (bertha-scf.f:150-611).
"""
import dataclasses
import math
import re

import numpy as np

from ._lib import HMLT, MAX_L, SHAPE


@dataclasses.dataclass
class Basis:
    xyz: np.ndarray            # [ncnt, 3] bohr
    lmax: np.ndarray           # [ncnt]
    nfn: np.ndarray            # [ncnt, MAX_L+1]
    ex: np.ndarray             # [ncnt, MAX_L+1, maxbs]
    hmlt: int = HMLT["DHFR"]
    isym: int = 0              # CLMFAST ISYM: 0 general, 1 linear, 2 atomic
    znuc: tuple = ()
    anuc: tuple = ()
    name: str = ""

    @property
    def ncnt(self):
        return int(self.xyz.shape[0])

    @property
    def nkap(self):
        return (2 * self.lmax + 1).astype(np.int32)

    @property
    def ndim(self):
        n = sum(4 * (2 * l + 1) * int(self.nfn[c, l])
                for c in range(self.ncnt) for l in range(int(self.lmax[c]) + 1))
        return n // 2 if self.hmlt == HMLT["NORL"] else n

    @property
    def nskp(self):
        return 0 if self.hmlt == HMLT["NORL"] else self.ndim // 2

    def shells(self):
        """Primitive shells (centre, l, ibas, exponent) in the library's order."""
        out = []
        for c in range(self.ncnt):
            for l in range(int(self.lmax[c]) + 1):
                for i in range(int(self.nfn[c, l])):
                    out.append((c, l, i, float(self.ex[c, l, i])))
        return out


def make_basis(centres, hmlt="DHFR", isym=None, name=""):
    """centres: list of (xyz, {l: exponents}) ; isym from the centre count
    and collinearity as NUCGEOM assigns SHAPE (bertha-scf.f:2150-2444)."""
    ncnt = len(centres)
    lmax = np.array([max(d.keys()) for _, d in centres], dtype=np.int32)
    if lmax.max() > MAX_L:
        raise ValueError(f"l > {MAX_L} is beyond the compiled limit")
    maxbs = max(len(v) for _, d in centres for v in d.values())
    nfn = np.zeros((ncnt, MAX_L + 1), dtype=np.int32)
    ex = np.zeros((ncnt, MAX_L + 1, maxbs))
    xyz = np.zeros((ncnt, 3))
    for c, (pos, d) in enumerate(centres):
        xyz[c] = pos
        for l, v in d.items():
            nfn[c, l] = len(v)
            ex[c, l, : len(v)] = v
    if isym is None:
        isym = shape_isym(xyz)
    return Basis(xyz=xyz, lmax=lmax, nfn=nfn, ex=ex, hmlt=HMLT[hmlt], isym=isym, name=name)


def shape_isym(xyz):
    """ISYM of CLMFAST from the SHAPE NUCGEOM would assign: ATOMIC for one
    centre, DIATOM for two, LINEAR when all centres share one axis, and
    NOSYMM otherwise (NUCGEOM overwrites PLANAR with NOSYMM, :2440-2444)."""
    n = len(xyz)
    if n == 1:
        return SHAPE["ATOMIC"]
    if n == 2:
        return SHAPE["DIATOM"]
    d = xyz - xyz[0]
    axis = d[np.argmax(np.linalg.norm(d, axis=1))]
    axis = axis / np.linalg.norm(axis)
    perp = d - np.outer(d @ axis, axis)
    return SHAPE["LINEAR"] if np.all(np.sum(perp ** 2, axis=1) < 1e-6) else SHAPE["NOSYMM"]


CFM = 5.29177211e4  # fm per bohr (bertha-scf.f:1013)
PRAD = 0.842        # proton rms charge radius, fm (bertha-scf.f:989)


def nuclear_exponents(znuc, anuc):
    """Gaussian nuclear exponents xi = 1.5/r_rms^2 (bohr^-2) of NUCCOUL
    (bertha-scf.f:1183-1210): r_rms = 0.842 fm for Z = 1, 0.836 A^(1/3) +
    0.57 fm for 1 < Z < 90, 0.770 A^(1/3) + 0.98 fm otherwise."""
    out = []
    for z, a in zip(znuc, anuc):
        if int(z) == 1:
            rfm = PRAD
        elif 1.0 < z < 90.0:
            rfm = 0.836 * a ** (1.0 / 3.0) + 0.57
        else:
            rfm = 0.770 * a ** (1.0 / 3.0) + 0.98
        r = rfm / CFM
        out.append(1.5 / (r * r))
    return np.array(out)


def geometric(alpha, beta, n):
    """Even-tempered exponents alpha*beta^k, k = 0..n-1 (CARDIN :361-387)."""
    return [alpha * beta ** k for k in range(n)]


def _tokens(line):
    out, s = [], line.strip()
    for m in re.finditer(r"'[^']*'|[^,\s]+", s):
        out.append(m.group(0).strip("'"))
    return out


def _num(tok):
    return float(tok.replace("D", "E").replace("d", "e"))


def read_deck(path):
    """Read a BERTHA .inp deck (CARDIN, bertha-scf.f:150-611) into a Basis.

    Supports the OPTIMISED, GEOMETRIC and EVENTEMPR basis types.  Returns
    (basis, meta) where meta holds the remaining fields: the calculation
    tree, NCLS (closed-shell spinors), the open-shell details of an
    open-shell deck (NOPN, NOELEC, ACFF, BCFF, IOPN; None when closed), the
    starting stage ILEV, READIN, the level shifts SHLEV(1..3) and each
    centre's electron count IQNC (the atomic configuration's, :313-314).
    """
    with open(path) as f:
        lines = [ln for ln in f.read().splitlines() if ln.strip()]
    it = iter(lines)

    def rec():
        return _tokens(next(it))

    rec(); molcl = rec()[0]
    rec(); tree = rec()[0]
    rec(); hmlt = rec()[0][:4]
    if hmlt not in HMLT:
        raise ValueError(f"unknown HMLT {hmlt}")
    rec(); readin = rec()[0].upper().startswith(".T")
    rec(); ncnt = int(rec()[0])
    centres, znuc, anuc, nelec = [], [], [], []
    for _ in range(ncnt):
        rec(); rec()
        pos = [_num(t) for t in rec()[:3]]
        rec(); nuc = rec()
        znuc.append(_num(nuc[1]))
        anuc.append(_num(nuc[2]) if len(nuc) > 2 else 2.0 * _num(nuc[1]))
        rec(); bt = rec()
        btyp, lmax = bt[0], int(bt[1])
        rec(); cnf = rec()
        nelec.append(int(_num(cnf[1])) if len(cnf) > 1 else int(round(znuc[-1])))
        if cnf[0] == "MANUAL":
            rec()
            for _l in range(lmax + 1):
                rec()
        rec()
        exps = {}
        for l in range(lmax + 1):
            if btyp == "OPTIMISED":
                n = int(rec()[0])
                exps[l] = [_num(rec()[0]) for _ in range(n)]
            elif btyp == "GEOMETRIC":
                t = rec()
                exps[l] = geometric(_num(t[0]), _num(t[1]), int(t[2]))
            elif btyp == "EVENTEMPR":
                t = rec()
                a, b, n, n1 = _num(t[0]), _num(t[1]), int(t[2]), int(t[3])
                exps[l] = geometric(a * b ** (n1 - 1), b, n)
            else:
                raise ValueError(f"illegal basis type {btyp}")
        centres.append((pos, exps))
    rec(); shl = rec()
    ncls = int(shl[0])
    nopn = int(shl[1]) if len(shl) > 1 else 0
    noelec = int(shl[2]) if len(shl) > 2 else 0
    open_shell = None
    title = rec()
    if nopn > 0:
        open_shell = {"nopn": nopn, "noelec": noelec, "acff": None, "bcff": None, "iopn": None}
        if "LEVEL SHIFT" not in " ".join(title).upper():
            # ACFF, BCFF and the open-shell orbitals IOPN (:486-489); older
            # decks go straight on to the level shifts
            t = rec()
            open_shell.update(acff=_num(t[0]), bcff=_num(t[1]),
                              iopn=[int(_num(x)) for x in t[2:2 + nopn]])
            title = rec()
    shifts = tuple(_num(t) for t in rec()[:3])
    rec(); ilev = int(rec()[0])
    basis = make_basis(centres, hmlt=hmlt, name=molcl)
    basis.znuc, basis.anuc = tuple(znuc), tuple(anuc)
    if hmlt == "NORL":
        ilev = 1
    if ncnt == 1 or readin:
        ilev = 3
    return basis, {"tree": tree, "ncls": ncls, "open_shell": open_shell, "ilev": ilev,
                   "readin": readin, "shifts": shifts, "nelec": tuple(nelec)}


# ---------------------------------------------------------------------------
# The workloads the benchmark is quoted on (synthetic, seeded)
# ---------------------------------------------------------------------------
def h2o_basis():
    """H2O: O 10s6p2d (0.10*2.8^k), H 6s2p (0.08*3.0^k); O at the origin,
    H at (+-1.430, 0, 1.107) bohr; Dirac-Coulomb."""
    o = {0: geometric(0.10, 2.8, 10), 1: geometric(0.10, 2.8, 6), 2: geometric(0.10, 2.8, 2)}
    h = {0: geometric(0.08, 3.0, 6), 1: geometric(0.08, 3.0, 2)}
    b = make_basis([((0, 0, 0), o), ((1.430, 0, 1.107), h), ((-1.430, 0, 1.107), h)],
                   hmlt="DHFR", name="H2O")
    b.znuc, b.anuc = (8.0, 1.0, 1.0), (16.0, 1.0, 1.0)
    return b


def tlf_basis():
    """TlF at R = 3.94 bohr on z: Tl 28s24p16d12f (0.02*2.2^k),
    F 14s9p3d (0.06*2.6^k); Dirac-Coulomb-Breit."""
    tl = {0: geometric(0.02, 2.2, 28), 1: geometric(0.02, 2.2, 24),
          2: geometric(0.02, 2.2, 16), 3: geometric(0.02, 2.2, 12)}
    f = {0: geometric(0.06, 2.6, 14), 1: geometric(0.06, 2.6, 9), 2: geometric(0.06, 2.6, 3)}
    b = make_basis([((0, 0, 0), tl), ((0, 0, 3.94), f)], hmlt="DHFB", name="TlF")
    b.znuc, b.anuc = (81.0, 9.0), (205.0, 19.0)
    return b


def tlf_small_basis():
    """TlF with the same geometry, angular momenta and exponent ranges as
    tlf_basis but few functions (Tl 7s6p4d3f, F 4s3p1d): a case that keeps
    TlF's quartet classes at about 1 % of its size (profiling, tests)."""
    tl = {0: geometric(0.02, 2.2 ** 4.5, 7), 1: geometric(0.02, 2.2 ** 4.6, 6),
          2: geometric(0.02, 2.2 ** 5.0, 4), 3: geometric(0.02, 2.2 ** 5.5, 3)}
    f = {0: geometric(0.06, 2.6 ** 4.3, 4), 1: geometric(0.06, 2.6 ** 4.0, 3), 2: [0.5]}
    b = make_basis([((0, 0, 0), tl), ((0, 0, 3.94), f)], hmlt="DHFB", name="TlF-small")
    b.znuc, b.anuc = (81.0, 9.0), (205.0, 19.0)
    return b


def c6h6_basis():
    """Benzene, planar D6h: C-C 2.637, C-H 2.048 bohr; C 14s9p4d2f
    (0.05*2.5^k), H 8s4p2d (0.07*2.8^k)."""
    c = {0: geometric(0.05, 2.5, 14), 1: geometric(0.05, 2.5, 9),
         2: geometric(0.05, 2.5, 4), 3: geometric(0.05, 2.5, 2)}
    h = {0: geometric(0.07, 2.8, 8), 1: geometric(0.07, 2.8, 4), 2: geometric(0.07, 2.8, 2)}
    cent = []
    for k in range(6):
        ang = math.pi / 3 * k
        u = np.array([math.cos(ang), math.sin(ang), 0.0])
        cent.append((2.637 * u, c))
    for k in range(6):
        ang = math.pi / 3 * k
        u = np.array([math.cos(ang), math.sin(ang), 0.0])
        cent.append(((2.637 + 2.048) * u, h))
    b = make_basis(cent, hmlt="DHFR", name="C6H6")
    b.znuc, b.anuc = (6.0,) * 6 + (1.0,) * 6, (12.0,) * 6 + (1.0,) * 6
    return b


# Atoms whose ground configuration fills every occupied subshell (closed
# shells from He to Rn), with the mass number of their most abundant isotope.
CLOSED_SHELL_ATOMS = {
    2: ("He", 4), 4: ("Be", 9), 10: ("Ne", 20), 12: ("Mg", 24), 18: ("Ar", 40),
    20: ("Ca", 40), 30: ("Zn", 64), 36: ("Kr", 84), 38: ("Sr", 88), 46: ("Pd", 106),
    48: ("Cd", 114), 54: ("Xe", 132), 56: ("Ba", 138), 70: ("Yb", 174), 80: ("Hg", 202),
    86: ("Rn", 222),
}


def atom_basis(z, hmlt="DHFR"):
    """Even-tempered closed-shell atom: n_s = 8 + Z/4, n_p = 6 + Z/5,
    n_d = Z/12, n_f = Z/24 functions (integer division), exponents
    0.03*2.4^k, one centre (ATOMIC); Gaussian nucleus of the most abundant
    isotope."""
    name, a = CLOSED_SHELL_ATOMS[int(z)]
    counts = (8 + z // 4, 6 + z // 5, z // 12, z // 24)
    exps = {l: geometric(0.03, 2.4, n) for l, n in enumerate(counts) if n > 0}
    b = make_basis([((0.0, 0.0, 0.0), exps)], hmlt=hmlt, name=name)
    b.znuc, b.anuc = (float(z),), (float(a),)
    return b


def batched_atoms(n=96, seed=2024, zset=None):
    """n closed-shell atoms with Z drawn uniformly (seeded) from zset
    (default: every closed-shell atom from He to Rn)."""
    zs = sorted(zset if zset is not None else CLOSED_SHELL_ATOMS)
    rng = np.random.default_rng(seed)
    return [atom_basis(int(z)) for z in rng.choice(zs, size=n)]


def density(basis, seed=0, nocc=None, real=False):
    """Seeded Hermitian positive semi-definite density D = C C^H (DENSTY
    form, bertha-scf.f:3600-3610) of nocc random orbitals."""
    rng = np.random.default_rng(seed)
    n = basis.ndim
    nocc = nocc or max(1, n // 8)
    C = rng.normal(size=(n, nocc))
    if not real:
        C = C + 1j * rng.normal(size=(n, nocc))
    C /= math.sqrt(n)
    D = np.conj(C) @ C.T
    return np.asfortranarray(D.astype(np.complex128))

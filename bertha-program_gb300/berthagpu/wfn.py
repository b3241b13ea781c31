"""Wavefunction files, the Fock layout and the atomic-density start.

``write_wfn``/``read_wfn`` keep the reference's `.wfn` file: NDIM records,
record I holding the eigenvalue EIGN(I) and the I-th eigenvector
COEF(1..NDIM, I), written list-directed (HFSCF, bertha-scf.f:5578-5583;
read back by CARDIN, :597-607).  ``density`` is DENSTY's closed-shell
density (:3580-3640) from such coefficients.  ``fock_layout`` restates
FOCKIND (:2582-2648), the order of the spinor basis in the Fock matrix,
which ``embed_atomic_densities`` uses to place atomic densities into a
molecule's matrix: the starting density of a molecular SCF built from SCFs
of its atoms (what the reference reads from bertha-atomic's files).
"""
import re

import numpy as np

from ._lib import HMLT, MAX_L

NKAP_SLOTS = 2 * MAX_L + 2   # KA = 1..2*LMAX+1 (1-based), as the C ABI's layout
NM_SLOTS = 28                # 2|m_j| - 1 + (m_j > 0)


def kappa_of(ka):
    """KAPA(KA) of CARDIN's kappa list: -1, 1, -2, 2, -3, 3, -4 (KA 1-based)."""
    if ka == 1:
        return -1
    return ka // 2 if ka % 2 == 0 else -(ka // 2) - 1


def lval(kappa):
    """LVAL (bertha-scf.f:21365): orbital l of a kappa."""
    return kappa if kappa > 0 else -kappa - 1


def fock_layout(basis):
    """FOCKIND: per centre, for |m_j| = 1/2, 3/2, ... the m_j < 0 blocks of
    every kappa with j >= |m_j| (in KA order), then the m_j > 0 blocks; each
    block holds the kappa's NFNC radial functions.  Returns (lrge, labels):
    lrge[centre, KA, 2|m_j|-1+(m_j>0)] = first large-component index (-1 if
    absent) and labels = int array [NSKP, 4] of (centre, kappa, 2 m_j, ibas)
    per large-component index.  The small components follow at +NSKP."""
    lrge = np.full((basis.ncnt, NKAP_SLOTS, NM_SLOTS), -1, dtype=np.int64)
    labels = []
    for c in range(basis.ncnt):
        nkap = int(basis.nkap[c])
        for imv in range(MAX_L + 1):
            mqn = 2 * imv + 1
            for sg in (0, 1):
                for ka in range(1, nkap + 1):
                    kq = kappa_of(ka)
                    if 2 * abs(kq) - 1 < mqn:
                        continue
                    nb = int(basis.nfn[c, lval(kq)])
                    lrge[c, ka, mqn - 1 + sg] = len(labels)
                    for i in range(nb):
                        labels.append((c, kq, mqn if sg else -mqn, i))
    return lrge, np.array(labels, dtype=np.int64).reshape(-1, 4)


def _fmt(x):
    return f"{x: .16E}"


def write_wfn(path, eign, coef):
    """EIGN(I), COEF(1..NDIM, I) per record, list-directed: reals as
    floating literals and complex values as (re,im), blank separated."""
    eign = np.asarray(eign, dtype=np.float64)
    coef = np.asarray(coef, dtype=np.complex128)
    n = coef.shape[0]
    if coef.shape != (n, n) or eign.shape != (n,):
        raise ValueError("write_wfn: need NDIM eigenvalues and an NDIM x NDIM COEF")
    with open(path, "w") as f:
        for i in range(n):
            parts = [_fmt(eign[i])]
            parts += [f"({_fmt(z.real)},{_fmt(z.imag)})" for z in coef[:, i]]
            f.write(" ".join(parts) + "\n")


_TOKEN = re.compile(r"\(\s*([^,()\s]+)\s*,\s*([^,()\s]+)\s*\)|([^\s,()]+)")


def _num(s):
    return float(s.replace("D", "E").replace("d", "e"))


def read_wfn(path, ndim):
    """Read an NDIM-record wavefunction file as CARDIN does (list-directed,
    so values may run across lines; `r*value` repeat counts are honoured).
    Returns (eign [NDIM], coef [NDIM, NDIM] with eigenvectors in columns)."""
    vals = []
    with open(path) as f:
        text = f.read()
    rep = 1  # a repeat count r* applies to the value that follows it
    for m in _TOKEN.finditer(text):
        if m.group(1) is not None:
            vals.extend([complex(_num(m.group(1)), _num(m.group(2)))] * rep)
            rep = 1
            continue
        tok = m.group(3)
        if "*" in tok:
            r, v = tok.split("*", 1)
            if not v:
                rep = int(r)
                continue
            vals.extend([complex(_num(v))] * int(r))
        else:
            vals.append(complex(_num(tok)))
        rep = 1
    need = ndim * (ndim + 1)
    if len(vals) < need:
        raise ValueError(f"read_wfn: {path} holds {len(vals)} values, {need} needed")
    arr = np.array(vals[:need], dtype=np.complex128).reshape(ndim, ndim + 1)
    return arr[:, 0].real.copy(), np.ascontiguousarray(arr[:, 1:].T)


def density(coef, nskp, nocc):
    """DENSTY (closed shells): D_ij = sum over the NOCC states above the NSKP
    negative-energy ones of conj(C_i) C_j."""
    occ = np.asarray(coef)[:, nskp:nskp + nocc]
    return np.conj(occ) @ occ.T


def atom_of_centre(basis, c, hmlt=None):
    """The one-centre basis of centre c (its exponents, at the origin)."""
    from .deck import make_basis
    lm = int(basis.lmax[c])
    exps = {l: [float(x) for x in basis.ex[c, l, :int(basis.nfn[c, l])]]
            for l in range(lm + 1) if basis.nfn[c, l] > 0}
    h = hmlt if hmlt is not None else [k for k, v in HMLT.items() if v == basis.hmlt][0]
    b = make_basis([((0.0, 0.0, 0.0), exps)], hmlt=h)
    b.znuc = (float(basis.znuc[c]),)
    b.anuc = (float(basis.anuc[c]),)
    return b


def centre_index_map(basis, c, atom):
    """Molecular Fock indices of the atom's spinor basis functions, in the
    atom's order (large components, then small ones at +NSKP)."""
    lm, _ = fock_layout(basis)
    la, labels_a = fock_layout(atom)
    nskp_m, nskp_a = basis.nskp, atom.nskp
    idx = np.empty(len(labels_a), dtype=np.int64)
    for k, (_, kq, m2, i) in enumerate(labels_a):
        ka = next(a for a in range(1, NKAP_SLOTS) if kappa_of(a) == kq)
        slot = abs(m2) - 1 + (m2 > 0)
        idx[k] = lm[c, ka, slot] + i
    if atom.hmlt == HMLT["NORL"]:
        return idx
    return np.concatenate([idx, idx + nskp_m]) if nskp_a else idx


def embed_atomic_densities(basis, atom_densities):
    """Superposition of atomic densities: atom_densities[c] (a density in the
    one-centre basis of centre c, or None) placed on centre c's block."""
    n = basis.ndim
    D = np.zeros((n, n), dtype=np.complex128)
    for c, Da in enumerate(atom_densities):
        if Da is None:
            continue
        idx = centre_index_map(basis, c, atom_of_centre(basis, c))
        D[np.ix_(idx, idx)] += np.asarray(Da)
    return D

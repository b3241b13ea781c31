"""One-centre Coulomb matrices by the reference's Racah route (test
infrastructure only: only tests/ import it, as a checker).

A restatement of COULOMB1 (bertha-scf.f:21540-22107) and the routines it
calls: TNSCLM1 (:25551) for the tensor orders allowed by the orbital
angular momenta, ANGCLM1 (:25865) with DK and SYM3J (:29166-29300) for the
angular factors, IJSET1/KLSET1 (:29301, :29394) for the normalisations and
exponent powers, BTACLM1 (:25380) for the beta integrals and RKCLM1
(:25664) for the radial integrals of the four component blocks, and the
closed-shell digestion of CLMMT1G (:24443): GDIR from (AB|CD) and GXCH
from (AD|CB).

The one-centre integrals of a single atom are formed for every ordering of
the four spinor labels; COULOMB1's permutation shortcuts (PRM1IJ, PRM1KL,
PRM1HC and CLMMT1G's reuse of each integral for its images) and the final
Hermitian completion are left out, so that the direct and exchange sums run
over whole matrices.  General shape (ISYM 0): no m selection beyond the
conservation rule m_a - m_b = m_d - m_c that CLMMT1G applies.  The MD
one-centre quartets that the GPU library uses when RACAH1 is off are
checked against this route.
"""
import math

import numpy as np

SENS = 1.0e-10   # COULOMB1's angular-factor cut (:21622)


def gamhlf(n):
    """GAMHLF(N) = Gamma(N/2) (GAMGEN, :1037)."""
    return math.gamma(n / 2.0)


def gamlog(n):
    """GAMLOG(N) = log Gamma(N/2) (GAMGEN)."""
    return math.lgamma(n / 2.0)


def sym3j(ja, l, jb, ma, m, mb):
    """Wigner 3j symbol (j l j'; m M m') with j = ja/2, j' = jb/2,
    m = ma/2, m' = mb/2 and l, M actual values (SYM3J, Racah's sum)."""
    if abs(m) > l or 2 * m + ma + mb != 0 or abs(ma) > ja or abs(mb) > jb:
        return 0.0
    t1, t2, t3 = (ja - jb) // 2 + l, (ja + jb) // 2 - l, (jb - ja) // 2 + l
    if min(t1, t2, t3) < 0:
        return 0.0
    f = math.factorial
    phs = (-1.0) ** ((ja - mb) // 2 - l)
    sym = math.sqrt(f((ja + ma) // 2) * f((ja - ma) // 2) * f((jb - mb) // 2)
                    * f((jb + mb) // 2) * f(l + m) * f(l - m))
    trp = math.sqrt(f(t1) * f(t2) * f(t3) / f((ja + jb) // 2 + l + 1))
    nui = max(l - (jb + ma) // 2, m + (ja - jb) // 2, 0)
    nuf = min((ja - ma) // 2, l + (ja - jb) // 2, l + m)
    x = 0.0
    for nu in range(nui, nuf + 1):
        x += (-1.0) ** nu / (f((ja - ma) // 2 - nu) * f((jb + ma) // 2 - l + nu)
                             * f((jb - ja) // 2 - m + nu) * f((ja - jb) // 2 + l - nu)
                             * f(l + m - nu) * f(nu))
    return phs * trp * sym * x


def dk(ja, ma, jb, mb, nu):
    """DK: angular coefficient of the Coulomb interaction at one vertex,
    order nu (twice-valued ja, ma, jb, mb)."""
    iq = (ma - mb) // 2
    phs = (-1.0) ** ((ma + 1) // 2)
    rtj = math.sqrt((ja + 1) * (jb + 1))
    return phs * rtj * sym3j(ja, nu, jb, 1, 0, -1) * sym3j(ja, nu, jb, -ma, iq, mb)


def tnsclm1(lqn):
    """Tensor orders NU of an LQN block (parity of both pairs even, triangle
    rules); empty when the block does not couple."""
    if (lqn[0] + lqn[1]) % 2 != (lqn[2] + lqn[3]) % 2:
        return []
    nui = max(abs(lqn[0] - lqn[1]), abs(lqn[2] - lqn[3]))
    nuf = min(lqn[0] + lqn[1], lqn[2] + lqn[3])
    return [nu for nu in range(nui, nuf + 1)
            if (lqn[0] + lqn[1] + nu) % 2 == 0 and (lqn[2] + lqn[3] + nu) % 2 == 0]


def angclm1(kqn, lqn, nus):
    """Surviving tensor orders of a KQN block and the angular factors
    DKAB[lten][(ma, mb)], DKCD[lten][(mc, md)] for signed twice-m values
    (ANGCLM1; DKCD with the arguments of the CD pair reversed)."""
    jq = [2 * abs(k) - 1 for k in kqn]
    nuit = max(abs(jq[0] - jq[1]) // 2, abs(jq[2] - jq[3]) // 2)
    nuft = min((jq[0] + jq[1]) // 2, (jq[2] + jq[3]) // 2)
    inu = [False] * len(nus)
    for nu in range(nuit, nuft + 1):
        if (lqn[0] + lqn[1] + nu) % 2 == 0 and (lqn[2] + lqn[3] + nu) % 2 == 0:
            inu[nus.index(nu)] = True
    if not any(inu):
        return None
    dkab, dkcd = {}, {}
    for lt, nu in enumerate(nus):
        if not inu[lt]:
            continue
        for ma in range(1, abs(kqn[0]) + 1):
            for mb in range(1, abs(kqn[1]) + 1):
                for sa in (-1, 1):
                    for sb in (-1, 1):
                        a, b = sa * (2 * ma - 1), sb * (2 * mb - 1)
                        dkab[(lt, a, b)] = dk(jq[0], a, jq[1], b, nu)
        for mc in range(1, abs(kqn[2]) + 1):
            for md in range(1, abs(kqn[3]) + 1):
                for sc in (-1, 1):
                    for sd in (-1, 1):
                        c, d = sc * (2 * mc - 1), sd * (2 * md - 1)
                        dkcd[(lt, c, d)] = dk(jq[3], d, jq[2], c, nu)
    return inu, dkab, dkcd


def _norms(l, ex):
    """IJSET1/KLSET1 normalisation constants (large, small) of radial
    functions r^l exp(-e r^2) of angular momentum l."""
    twlg = math.log(2.0)
    g1, g2 = twlg - gamlog(2 * l + 3), twlg - gamlog(2 * l + 5)
    el = np.log(2.0 * ex)
    return np.exp(0.5 * (g1 + (l + 1.5) * el)), np.exp(0.5 * (g2 + (l + 0.5) * el))


def _beta(xj, ia, ib):
    """BTACLM1's incomplete beta integral for arguments xj (array)."""
    if ib > 1:
        x = ia + 0.5
        bta1 = np.sqrt(xj) ** (2 * ia + 1) / x
        ra, rb, rc, rd = x, float(1 - ib), x + 1.0, 1.0
        trm = ra * rb / (rc * rd) * xj
        binv = 1.0 + trm
        ra, rb, rc, rd = ra + 1.0, rb + 1.0, rc + 1.0, rd + 1.0
        for _ in range(2, ib):
            trm = ra * rb / (rc * rd) * trm * xj
            binv = binv + trm
            ra, rb, rc, rd = ra + 1.0, rb + 1.0, rc + 1.0, rd + 1.0
        return bta1 * binv
    if ib == 1:
        return np.sqrt(xj) ** (2 * ia + 1) / (ia + 0.5)
    xr = np.sqrt(xj)
    bta1 = np.log((1.0 + xr) / (1.0 - xr))
    if ia > 1:
        binv = np.ones_like(xj)
        trm = xj.copy()
        for k in range(2, ia + 1):
            binv = binv + trm / (2 * k - 1)
            trm = trm * xj
        return bta1 - 2.0 * xr * binv
    if ia == 1:
        return bta1 - 2.0 * xr
    return bta1


def rk_block(kqn, lqn, nus, inu, exps):
    """RKCLM1 (with IJSET1, KLSET1, BTACLM1) for every exponent quadruple of
    a KQN block: radial integrals RJ[component][lten] as arrays
    [na, nb, nc, nd], components LLLL, LLSS, SSLL, SSSS, normalised."""
    ea, eb, ec, ed = (np.asarray(e, dtype=float) for e in exps)
    EI, EJ = np.meshgrid(ea, eb, indexing="ij")
    EK, EL = np.meshgrid(ec, ed, indexing="ij")
    EI, EJ = EI[:, :, None, None], EJ[:, :, None, None]
    EK, EL = EK[None, None, :, :], EL[None, None, :, :]
    tij0, tkl0 = EI + EJ, EK + EL
    xj = (np.broadcast_to(tij0 / (tij0 + tkl0), (len(ea), len(eb), len(ec), len(ed))),
          np.broadcast_to(tkl0 / (tij0 + tkl0), (len(ea), len(eb), len(ec), len(ed))))
    nui, nuf = nus[0], nus[-1]
    nunum = len(nus)
    nvals = (nuf - nui) // 2 + 3
    bdu, bdl = {}, {}
    for nx in range(1, nvals + 1):
        iaa = (lqn[0] + lqn[1] + nui + 2 * nx - 1, lqn[2] + lqn[3] + nui + 2 * nx - 1)
        for ny in range(1, nvals + 1):
            ibb = (lqn[2] + lqn[3] - nuf + 2 * ny - 2, lqn[0] + lqn[1] - nuf + 2 * ny - 2)
            bdu[(nx, ny)] = _beta(xj[0], (iaa[0] - 1) // 2, ibb[0] // 2)
            bdl[(nx, ny)] = _beta(xj[1], (iaa[1] - 1) // 2, ibb[1] // 2)
    # EIJ(p) = (EI + EJ)^(-(LA + LB + p)/2), EKL likewise (IJSET1/KLSET1)
    def eij(p):
        return np.sqrt(tij0) ** (-(lqn[0] + lqn[1] + p))

    def ekl(p):
        return np.sqrt(tkl0) ** (-(lqn[2] + lqn[3] + p))
    lsum = sum(lqn)
    C1, C3, C5, C7, C9 = (0.25 * gamhlf(lsum + k) for k in (1, 3, 5, 7, 9))
    ti, tj, tk, tl = (float(lqn[n] + kqn[n] + 1) for n in range(4))
    out = {c: [None] * nunum for c in ("LLLL", "LLSS", "SSLL", "SSSS")}
    for lt in range(nunum):
        if not inu[lt]:
            continue
        nten = nunum - (lt + 1)
        nu = nus[lt]
        L = lt + 1   # 1-based LTEN of the reference
        B10 = eij(-nu) * ekl(nu + 1) * bdl[(L, nten + 1)] + eij(nu + 1) * ekl(-nu) * bdu[(L, nten + 1)]
        B12 = eij(-nu + 2) * ekl(nu + 1) * bdl[(L, nten + 2)] + eij(nu + 3) * ekl(-nu) * bdu[(L + 1, nten + 1)]
        B14 = eij(-nu + 4) * ekl(nu + 1) * bdl[(L, nten + 3)] + eij(nu + 5) * ekl(-nu) * bdu[(L + 2, nten + 1)]
        B30 = eij(-nu) * ekl(nu + 3) * bdl[(L + 1, nten + 1)] + eij(nu + 1) * ekl(-nu + 2) * bdu[(L, nten + 2)]
        B32 = eij(-nu + 2) * ekl(nu + 3) * bdl[(L + 1, nten + 2)] + eij(nu + 3) * ekl(-nu + 2) * bdu[(L + 1, nten + 2)]
        B34 = eij(-nu + 4) * ekl(nu + 3) * bdl[(L + 1, nten + 3)] + eij(nu + 5) * ekl(-nu + 2) * bdu[(L + 2, nten + 2)]
        B50 = eij(-nu) * ekl(nu + 5) * bdl[(L + 2, nten + 1)] + eij(nu + 1) * ekl(-nu + 4) * bdu[(L, nten + 3)]
        B52 = eij(-nu + 2) * ekl(nu + 5) * bdl[(L + 2, nten + 2)] + eij(nu + 3) * ekl(-nu + 4) * bdu[(L + 1, nten + 3)]
        B54 = eij(-nu + 4) * ekl(nu + 5) * bdl[(L + 2, nten + 3)] + eij(nu + 5) * ekl(-nu + 4) * bdu[(L + 2, nten + 3)]
        out["LLLL"][lt] = C5 * B32
        out["LLSS"][lt] = (4 * EK * EL * C7 * B52 - 2 * tl * EK * C5 * B32
                           - 2 * tk * EL * C5 * B32 + tk * tl * C3 * B12)
        out["SSLL"][lt] = (4 * EI * EJ * C7 * B34 - 2 * tj * EI * C5 * B32
                           - 2 * ti * EJ * C5 * B32 + ti * tj * C3 * B30)
        out["SSSS"][lt] = (16 * EI * EJ * EK * EL * C9 * B54
                           - 8 * tl * EI * EJ * EK * C7 * B34 - 8 * tk * EI * EJ * EL * C7 * B34
                           - 8 * tj * EI * EK * EL * C7 * B52 - 8 * ti * EJ * EK * EL * C7 * B52
                           + 4 * ti * tj * EK * EL * C5 * B50 + 4 * tk * tl * EI * EJ * C5 * B14
                           + 4 * ti * tl * EJ * EK * C5 * B32 + 4 * tj * tk * EI * EL * C5 * B32
                           + 4 * tj * tl * EI * EK * C5 * B32 + 4 * ti * tk * EJ * EL * C5 * B32
                           - 2 * ti * tj * tl * EK * C3 * B30 - 2 * tj * tk * tl * EI * C3 * B12
                           - 2 * ti * tj * tk * EL * C3 * B30 - 2 * ti * tk * tl * EJ * C3 * B12
                           + ti * tj * tk * tl * C1 * B10)
    nla, nsa = _norms(lqn[0], ea)
    nlb, nsb = _norms(lqn[1], eb)
    nlc, nsc = _norms(lqn[2], ec)
    nld, nsd = _norms(lqn[3], ed)
    rn = {"L": (nla[:, None] * nlb[None, :], nlc[:, None] * nld[None, :]),
          "S": (nsa[:, None] * nsb[None, :], nsc[:, None] * nsd[None, :])}
    for comp in out:
        fab = rn[comp[0]][0][:, :, None, None]
        fcd = rn[comp[2]][1][None, None, :, :]
        out[comp] = [None if x is None else x * fab * fcd for x in out[comp]]
    return out


def kappa_of(ka):
    """KAPA(KA): -1, 1, -2, 2, -3, 3, -4 for KA = 1, 2, ... (CARDIN)."""
    if ka == 1:
        return -1
    return ka // 2 if ka % 2 == 0 else -(ka // 2) - 1


def coulomb1(basis, dent, lrge, pairs=None):
    """GDIR and GXCH (full NDIM x NDIM) of a one-centre basis (centre 0)
    for the density DENT, by COULOMB1's Racah route; lrge[0, KA, slot] is
    the first large-component Fock index of the (KA, m) block, slot =
    2|m| - 1 + (m > 0) - 1 (FOCKIND).  pairs: only these (KA, KB) blocks
    (the contributions of disjoint sets of pairs add up to the whole)."""
    n = dent.shape[0]
    nskp = n // 2
    gd = np.zeros((n, n), dtype=complex)
    gx = np.zeros((n, n), dtype=complex)
    lmax = int(basis.lmax[0])
    nkap = 2 * lmax + 1
    kas = list(range(1, nkap + 1))
    exps = {l: np.asarray(basis.ex[0, l, :int(basis.nfn[0, l])], dtype=float)
            for l in range(lmax + 1)}

    def lv(k):
        return k if k > 0 else -k - 1

    def blk(ka, m2):
        """Large-component index range of spinors (KA, m = m2/2)."""
        k = kappa_of(ka)
        slot = abs(m2) - 1 + (1 if m2 > 0 else 0)
        o = int(lrge[0, ka, slot])
        return o, o + len(exps[lv(k)])

    for ka in kas:
        for kb in kas:
            if pairs is not None and (ka, kb) not in pairs:
                continue
            for kc in kas:
                for kd in kas:
                    kqn = [kappa_of(k) for k in (ka, kb, kc, kd)]
                    lqn = [lv(k) for k in kqn]
                    nus = tnsclm1(lqn)
                    if not nus:
                        continue
                    ang = angclm1(kqn, lqn, nus)
                    if ang is None:
                        continue
                    inu, dkab, dkcd = ang
                    rj = rk_block(kqn, lqn, nus, inu, [exps[l] for l in lqn])
                    ms = [[s * (2 * m - 1) for m in range(1, abs(k) + 1) for s in (-1, 1)]
                          for k in kqn]
                    for ma in ms[0]:
                        for mb in ms[1]:
                            for mc in ms[2]:
                                for md in ms[3]:
                                    if ma - mb != md - mc:
                                        continue
                                    X = {}
                                    for comp in rj:
                                        acc = 0.0
                                        for lt in range(len(nus)):
                                            if not inu[lt]:
                                                continue
                                            f = dkab[(lt, ma, mb)] * dkcd[(lt, mc, md)]
                                            if abs(f) <= SENS:
                                                continue
                                            acc = acc + f * rj[comp][lt]
                                        X[comp] = acc
                                    if all(np.isscalar(v) for v in X.values()):
                                        continue
                                    a0, a1 = blk(ka, ma)
                                    b0, b1 = blk(kb, mb)
                                    c0, c1 = blk(kc, mc)
                                    d0, d1 = blk(kd, md)
                                    L = {"a": slice(a0, a1), "b": slice(b0, b1),
                                         "c": slice(c0, c1), "d": slice(d0, d1)}
                                    S = {k: slice(v.start + nskp, v.stop + nskp)
                                         for k, v in L.items()}
                                    XL4, XLS, XSL, XS4 = (X[c] for c in ("LLLL", "LLSS", "SSLL",
                                                                         "SSSS"))
                                    # GDIR: (AB|CD)
                                    gd[L["a"], L["b"]] += (
                                        np.einsum("abcd,cd->ab", XL4, dent[L["c"], L["d"]])
                                        + np.einsum("abcd,cd->ab", XLS, dent[S["c"], S["d"]]))
                                    gd[S["a"], S["b"]] += (
                                        np.einsum("abcd,cd->ab", XSL, dent[L["c"], L["d"]])
                                        + np.einsum("abcd,cd->ab", XS4, dent[S["c"], S["d"]]))
                                    # GXCH: (AD|CB)
                                    gx[L["a"], L["d"]] += np.einsum("abcd,cb->ad", XL4,
                                                                    dent[L["c"], L["b"]])
                                    gx[S["a"], S["d"]] += np.einsum("abcd,cb->ad", XS4,
                                                                    dent[S["c"], S["b"]])
                                    gx[L["a"], S["d"]] += np.einsum("abcd,cb->ad", XLS,
                                                                    dent[S["c"], L["b"]])
                                    gx[S["a"], L["d"]] += np.einsum("abcd,cb->ad", XSL,
                                                                    dent[L["c"], S["b"]])
    return gd, gx


# ---------------------------------------------------------------------------
# One-centre Breit (Gaunt plus gauge) exchange matrix by the Racah route:
# BREIT1 (bertha-scf.f:26014) with TNSBRT1 (:28691), ANGBRT1 (:28813),
# BRCOEF1 (the coefficients of Grant and Pyper's table 2), BTABRT1 (:28354),
# RKBRT1 (:28525) and the closed-shell exchange digestion of BRTMT1G
# (:27462): BXCH from (AD|CB).
# ---------------------------------------------------------------------------

def tnsbrt1(lqn):
    """Tensor orders of the Breit interaction for an LQN block: NU where
    both LA+LB+NU and LC+LD+NU are odd (NU > 0), NU-1 and NU+1 where both
    are even (NU-1 only for NU > 0); an ordered list without repeats."""
    if (lqn[0] + lqn[1]) % 2 != (lqn[2] + lqn[3]) % 2:
        return []
    nui = max(abs(lqn[0] - lqn[1]), abs(lqn[2] - lqn[3]))
    nuf = min(lqn[0] + lqn[1], lqn[2] + lqn[3])
    if nui > nuf:
        return []
    out = []
    for nu in range(nui, nuf + 1):
        pab, pcd = (lqn[0] + lqn[1] + nu) % 2, (lqn[2] + lqn[3] + nu) % 2
        if pab == 1 and pcd == 1 and nu != 0:
            vals = [nu]
        elif pab == 0 and pcd == 0:
            vals = ([nu - 1] if nu > 0 else []) + [nu + 1]
        else:
            vals = []
        for v in vals:
            if v not in out:
                out.append(v)
    return sorted(out)


def brcoef1(kqn, nu):
    """SCOEFF[i][0] (order NU-1) and SCOEFF[i][1] (order NU+1) for the eight
    component integrals LSLS, SLSL, LSSL, SLLS (upper, lower) (BRCOEF1)."""
    kca, kdb = kqn[1] - kqn[0], kqn[3] - kqn[2]
    s = [[0.0, 0.0] for _ in range(8)]
    if nu >= 1:
        b1 = nu * (nu + 1) / (2 * nu * (2 * nu - 1))
        c1 = (nu - 2) / (2 * nu * (2 * nu - 1))
        s[0][0] = (nu + kca) * (b1 - c1 * kdb)
        s[1][0] = (nu + kdb) * (b1 - c1 * kca)
        s[2][0] = (nu - kca) * (b1 + c1 * kdb)
        s[3][0] = (nu - kdb) * (b1 + c1 * kca)
        s[4][0] = -(nu + kca) * (b1 + c1 * kdb)
        s[5][0] = -(nu - kdb) * (b1 - c1 * kca)
        s[6][0] = -(nu - kca) * (b1 - c1 * kdb)
        s[7][0] = -(nu + kdb) * (b1 + c1 * kca)
    if nu >= 0:
        b2 = nu * (nu + 1) / ((2 * nu + 2) * (2 * nu + 3))
        c2 = (nu + 3) / ((2 * nu + 2) * (2 * nu + 3))
        s[0][1] = -(nu + 1 - kdb) * (b2 + c2 * kca)
        s[1][1] = -(nu + 1 - kca) * (b2 + c2 * kdb)
        s[2][1] = -(nu + 1 + kdb) * (b2 - c2 * kca)
        s[3][1] = -(nu + 1 + kca) * (b2 - c2 * kdb)
        s[4][1] = (nu + 1 + kdb) * (b2 + c2 * kca)
        s[5][1] = (nu + 1 - kca) * (b2 - c2 * kdb)
        s[6][1] = (nu + 1 - kdb) * (b2 - c2 * kca)
        s[7][1] = (nu + 1 + kca) * (b2 + c2 * kdb)
    return s


def angbrt1(kqn, lqn, nus):
    """Breit angular coefficients BCOF[lten][imu] as dicts over the signed
    twice-m values (ma, mb, mc, md), and the flags of the orders used by
    this KQN block (ANGBRT1)."""
    jq = [2 * abs(k) - 1 for k in kqn]
    nuit = max(abs(jq[0] - jq[1]) // 2, abs(jq[2] - jq[3]) // 2)
    nuft = min((jq[0] + jq[1]) // 2, (jq[2] + jq[3]) // 2)
    if nuit > nuft:
        return None
    if (lqn[0] + lqn[1]) % 2 != (lqn[2] + lqn[3]) % 2:
        return None
    mss = [[s * (2 * m - 1) for m in range(1, abs(k) + 1) for s in (-1, 1)] for k in kqn]
    inu = [False] * len(nus)
    bcof = [[{} for _ in range(8)] for _ in nus]
    used = False

    def add(lt, coef):
        # BCOF(lt, imu, ...) += AJJN * coef[imu]
        for imu in range(8):
            c = coef[imu]
            if c == 0.0:
                continue
            d = bcof[lt][imu]
            for key, v in ajjn.items():
                d[key] = d.get(key, 0.0) + v * c
    for nu in range(nuit, nuft + 1):
        pab, pcd = (lqn[0] + lqn[1] + nu) % 2, (lqn[2] + lqn[3] + nu) % 2
        if not ((pab == 1 and pcd == 1 and nu != 0) or (pab == 0 and pcd == 0)):
            continue
        ajjn = {}
        for ma in mss[0]:
            for mb in mss[1]:
                dab = dk(jq[0], ma, jq[1], mb, nu)
                for mc in mss[2]:
                    for md in mss[3]:
                        ajjn[(ma, mb, mc, md)] = dab * dk(jq[3], md, jq[2], mc, nu)
        used = True
        if pab == 1:
            lt = nus.index(nu)
            inu[lt] = True
            rc = -(kqn[0] + kqn[1]) * (kqn[2] + kqn[3]) / (nu * (nu + 1))
            add(lt, [rc] * 8)
        else:
            sc = brcoef1(kqn, nu)
            if nu > 0:
                lt = nus.index(nu - 1)
                inu[lt] = True
                add(lt, [sc[i][0] for i in range(8)])
            lt = nus.index(nu + 1)
            inu[lt] = True
            add(lt, [sc[i][1] for i in range(8)])
    if not used:
        return None
    return inu, bcof


def rk_breit_block(kqn, lqn, nus, inu, exps):
    """RKBRT1 (with IJSET1, KLSET1, BTABRT1): radial Breit integrals
    RJ[comp][lten] = (upper, lower) arrays [na, nb, nc, nd] for the
    component integrals LSLS, SLSL, LSSL, SLLS, normalised."""
    ea, eb, ec, ed = (np.asarray(e, dtype=float) for e in exps)
    shp = (len(ea), len(eb), len(ec), len(ed))
    EI = ea[:, None, None, None] * np.ones(shp)
    EJ = eb[None, :, None, None] * np.ones(shp)
    EK = ec[None, None, :, None] * np.ones(shp)
    EL = ed[None, None, None, :] * np.ones(shp)
    tij0, tkl0 = EI + EJ, EK + EL
    xj = (tij0 / (tij0 + tkl0), tkl0 / (tij0 + tkl0))
    nui, nuf = nus[0], nus[-1]
    nunum = len(nus)
    nvals = (nuf - nui) // 2 + 2
    bdu, bdl = {}, {}
    for nx in range(1, nvals + 1):
        iaa = (lqn[0] + lqn[1] + nui + 2 * nx, lqn[2] + lqn[3] + nui + 2 * nx)
        for ny in range(1, nvals + 1):
            ibb = (lqn[2] + lqn[3] - nuf + 2 * ny - 1, lqn[0] + lqn[1] - nuf + 2 * ny - 1)
            bdu[(nx, ny)] = _beta(xj[0], (iaa[0] - 1) // 2, ibb[0] // 2)
            bdl[(nx, ny)] = _beta(xj[1], (iaa[1] - 1) // 2, ibb[1] // 2)

    def eij(p):
        return np.sqrt(tij0) ** (-(lqn[0] + lqn[1] + p))

    def ekl(p):
        return np.sqrt(tkl0) ** (-(lqn[2] + lqn[3] + p))
    lsum = sum(lqn)
    C3, C5, C7 = (0.25 * gamhlf(lsum + k) for k in (3, 5, 7))
    ti, tj, tk, tl = (float(lqn[n] + kqn[n] + 1) for n in range(4))
    out = {c: [None] * nunum for c in ("LSLS", "SLSL", "LSSL", "SLLS")}
    for lt in range(nunum):
        if not inu[lt]:
            continue
        L, nten, nu = lt + 1, nunum - (lt + 1), nus[lt]
        B21L = eij(-nu + 1) * ekl(nu + 2) * bdl[(L, nten + 1)]
        B21U = eij(nu + 2) * ekl(-nu + 1) * bdu[(L, nten + 1)]
        B23L = eij(-nu + 3) * ekl(nu + 2) * bdl[(L, nten + 2)]
        B41U = eij(nu + 4) * ekl(-nu + 1) * bdu[(L + 1, nten + 1)]
        B41L = eij(-nu + 1) * ekl(nu + 4) * bdl[(L + 1, nten + 1)]
        B23U = eij(nu + 2) * ekl(-nu + 3) * bdu[(L, nten + 2)]
        B43L = eij(-nu + 3) * ekl(nu + 4) * bdl[(L + 1, nten + 2)]
        B43U = eij(nu + 4) * ekl(-nu + 3) * bdu[(L + 1, nten + 2)]

        def pair(E1, E2, T1, T2):
            # (4 E1 E2 C7 B43 - 2 T2 E1 C5 B41 - 2 T1 E2 C5 B23 + T1 T2 C3 B21),
            # upper; the lower form swaps B41 and B23
            up = (4 * E1 * E2 * C7 * B43U - 2 * T2 * E1 * C5 * B41U
                  - 2 * T1 * E2 * C5 * B23U + T1 * T2 * C3 * B21U)
            lo = (4 * E1 * E2 * C7 * B43L - 2 * T2 * E1 * C5 * B23L
                  - 2 * T1 * E2 * C5 * B41L + T1 * T2 * C3 * B21L)
            return up, lo
        out["LSLS"][lt] = pair(EJ, EL, tj, tl)
        out["SLSL"][lt] = pair(EI, EK, ti, tk)
        out["LSSL"][lt] = pair(EJ, EK, tj, tk)
        out["SLLS"][lt] = pair(EI, EL, ti, tl)
    nla, nsa = _norms(lqn[0], ea)
    nlb, nsb = _norms(lqn[1], eb)
    nlc, nsc = _norms(lqn[2], ec)
    nld, nsd = _norms(lqn[3], ed)
    N = {"L": (nla, nlb, nlc, nld), "S": (nsa, nsb, nsc, nsd)}
    for comp in out:
        f = (N[comp[0]][0][:, None, None, None] * N[comp[1]][1][None, :, None, None]
             * N[comp[2]][2][None, None, :, None] * N[comp[3]][3][None, None, None, :])
        out[comp] = [None if x is None else (x[0] * f, x[1] * f) for x in out[comp]]
    return out


def breit1(basis, dent, lrge):
    """BXCH (full NDIM x NDIM) of a one-centre basis (centre 0) for the
    density DENT by BREIT1's Racah route (Gaunt plus gauge term)."""
    n = dent.shape[0]
    nskp = n // 2
    bx = np.zeros((n, n), dtype=complex)
    lmax = int(basis.lmax[0])
    kas = list(range(1, 2 * lmax + 2))
    exps = {l: np.asarray(basis.ex[0, l, :int(basis.nfn[0, l])], dtype=float)
            for l in range(lmax + 1)}

    def lv(k):
        return k if k > 0 else -k - 1

    def rng(ka, m2, comp):
        k = kappa_of(ka)
        o = int(lrge[0, ka, abs(m2) - 1 + (1 if m2 > 0 else 0)])
        if comp == "S":
            o += nskp
        return slice(o, o + len(exps[lv(k)]))
    icomp = {"LSLS": 0, "SLSL": 2, "LSSL": 4, "SLLS": 6}
    for ka in kas:
        for kb in kas:
            for kc in kas:
                for kd in kas:
                    kqn = [kappa_of(k) for k in (ka, kb, kc, kd)]
                    lqn = [lv(k) for k in kqn]
                    nus = tnsbrt1(lqn)
                    if not nus:
                        continue
                    ang = angbrt1(kqn, lqn, nus)
                    if ang is None:
                        continue
                    inu, bcof = ang
                    rj = rk_breit_block(kqn, lqn, nus, inu, [exps[l] for l in lqn])
                    ms = [[s * (2 * m - 1) for m in range(1, abs(k) + 1) for s in (-1, 1)]
                          for k in kqn]
                    for ma in ms[0]:
                        for mb in ms[1]:
                            for mc in ms[2]:
                                for md in ms[3]:
                                    if ma - md != mb - mc:
                                        continue
                                    key = (ma, mb, mc, md)
                                    X = {}
                                    for comp, i0 in icomp.items():
                                        acc = 0.0
                                        for lt in range(len(nus)):
                                            if not inu[lt]:
                                                continue
                                            fu = bcof[lt][i0].get(key, 0.0)
                                            fl = bcof[lt][i0 + 1].get(key, 0.0)
                                            angsum = sum(abs(bcof[lt][i].get(key, 0.0))
                                                         for i in range(8))
                                            if angsum <= SENS:
                                                continue
                                            up, lo = rj[comp][lt]
                                            acc = acc + fu * up + fl * lo
                                        X[comp] = acc
                                    for comp, x in X.items():
                                        if np.isscalar(x):
                                            continue
                                        ta, tb, tc, td = comp
                                        # BXCH: (AD|CB), K(a, d) += (ab|cd) D(c, b)
                                        bx[rng(ka, ma, ta), rng(kd, md, td)] += np.einsum(
                                            "abcd,cb->ad", x, dent[rng(kc, mc, tc), rng(kb, mb, tb)])
    return bx

"""CPU-side checks: the C-ABI library loads and exports every declared
symbol; host-side basis layout agrees with the oracle's FOCKIND."""
import ctypes
import os
import re

import numpy as np
import pytest

import berthagpu
from berthagpu import _lib, deck
from berthagpu.build import build as build_lib
from oracle import oracle as orc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    hdr = open(os.path.join(ROOT, "include", "bertha_gpu.h")).read()
    return sorted(set(re.findall(r"\b(bertha_gpu_\w+)\s*\(", hdr)))


def test_library_exports_all_declared_symbols():
    path = build_lib()
    L = ctypes.CDLL(path)
    names = _declared()
    assert names, "no declarations found"
    for n in names:
        assert hasattr(L, n), n
    assert sorted(_lib.EXPORTED) == names


def test_ndim_matches_oracle_layout():
    for b in (deck.h2o_basis(), deck.tlf_basis()):
        ndim, nskp, lrge = orc.fock_layout(b)
        assert ndim == b.ndim and nskp == b.nskp


def test_fock_layout_is_a_permutation():
    b = deck.h2o_basis()
    ndim, nskp, lrge = orc.fock_layout(b)
    seen = np.zeros(nskp, int)
    for c in range(b.ncnt):
        for l in range(int(b.lmax[c]) + 1):
            n = int(b.nfn[c, l])
            for ka in ([1] if l == 0 else [2 * l, 2 * l + 1]):
                kq = -1 if ka == 1 else (ka // 2 if ka % 2 == 0 else -(ka // 2) - 1)
                for m in range(2 * abs(kq)):
                    base = lrge[c, ka, m]
                    assert base >= 0
                    seen[base:base + n] += 1
    assert np.all(seen == 1)


def test_deck_reader_reference_format(tmp_path):
    text = """'OUTPUT STRING'
HF2
'CALCULATION TREE'
HFSCF
'HAMILTONIAN'
DHFR
'CONTINUING'
.FALSE.
'NUMBER OF ATOMIC CENTRES'
2
'CENTER 1'
'CARTESIAN COORDINATES'
0.0,0.0,0.0
'NUCLEUS'
GAUSS,1,1.0000
'ATOMIC BASIS: TYPE AND LMAX'
GEOMETRIC,1
'ELECTRON CONFIGURATION'
AUFBAU,1
'BASIS SET EXPONENTS'
0.1,2.0,3
0.2,3.0,2
'CENTER 2'
'CARTESIAN COORDINATES'
0.0,0.0,1.4
'NUCLEUS'
GAUSS,9,19.0
'ATOMIC BASIS: TYPE AND LMAX'
OPTIMISED,0
'ELECTRON CONFIGURATION'
AUFBAU,9
'BASIS SET EXPONENTS'
2
1.5D+01
3.0D-01
'CLOSED/OPEN'
10,0,0
'LEVEL SHIFT'
1.0,1.0,0.5
'STARTING STAGE'
1
"""
    p = tmp_path / "hf.inp"
    p.write_text(text)
    b, meta = deck.read_deck(str(p))
    assert b.ncnt == 2 and b.isym == 1
    assert np.allclose(b.ex[0, 0, :3], [0.1, 0.2, 0.4])
    assert np.allclose(b.ex[0, 1, :2], [0.2, 0.6])
    assert np.allclose(b.ex[1, 0, :2], [15.0, 0.3])
    assert meta["ilev"] == 1 and meta["ncls"] == 10
    assert meta["shifts"] == (1.0, 1.0, 0.5) and meta["nelec"] == (1, 9)
    assert b.ndim == 4 * (3 + 3 * 2) + 4 * 2


def test_deck_reader_open_shell(tmp_path):
    """NOPN > 0: ACFF, BCFF and IOPN follow (:486-489), or, in older
    decks, the level shifts follow directly."""
    head = """'OUTPUT STRING'
Cs
'TREE'
HFSCF
'HAMILTONIAN'
DHFR
'CONTINUING'
.FALSE.
'NUMBER OF ATOMIC CENTRES'
1
'CENTER 1'
'CARTESIAN COORDINATES'
0.0,0.0,0.0
'NUCLEUS'
GAUSS,55,132.9
'ATOMIC BASIS: TYPE AND LMAX'
GEOMETRIC,1
'ELECTRON CONFIGURATION'
AUFBAU,55
'BASIS SET EXPONENTS'
0.01 2.1 30
0.01 2.1 20
'NUMBER OF CLOSED- AND OPEN-SHELL ORBITALS AND OPEN-SHELL ELECTRONS'
54,2,1
"""
    tail = """'LEVEL SHIFT PARAMETER FOR EACH INTEGRAL INCLUSION LEVEL'
0.3,0.3,0.2
'STARTING STAGE'
1
"""
    new = head + "'SPECIFY OPEN-SHELL INFORMATION'\n0.0D0,-2.0D0,55,56\n" + tail
    for text, iopn in ((new, [55, 56]), (head + tail, None)):
        p = tmp_path / "cs.inp"
        p.write_text(text)
        b, meta = deck.read_deck(str(p))
        assert meta["ncls"] == 54 and meta["shifts"] == (0.3, 0.3, 0.2)
        o = meta["open_shell"]
        assert o["nopn"] == 2 and o["noelec"] == 1 and o["iopn"] == iopn
        assert b.nfn[0, 0] == 30 and abs(b.ex[0, 0, 29] - 0.01 * 2.1 ** 29) < 1e-6


def test_missing_library_fails_loudly(monkeypatch):
    monkeypatch.setattr(_lib, "_L", None)
    monkeypatch.setattr(_lib, "LIB", "/nonexistent/libberthagpu.so")
    with pytest.raises(berthagpu.BerthaGPUError):
        _lib.lib()

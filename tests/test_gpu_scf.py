"""DHF SCF on the GPU (device Fock builds, one-electron matrices, cuSOLVER
eigensolver through torch) against the same loop on the oracle backend."""
import pytest

pytestmark = pytest.mark.gpu

import torch  # noqa: E402

from berthagpu import deck  # noqa: E402
from berthagpu.scf import DHFSCF  # noqa: E402
from scf_oracle import OracleBackend  # noqa: E402


def _water_small(hmlt="DHFR"):
    o = {0: deck.geometric(0.15, 3.5, 6), 1: deck.geometric(0.2, 3.5, 3)}
    h = {0: deck.geometric(0.1, 3.5, 3)}
    b = deck.make_basis([((0, 0, 0), o), ((1.430, 0, 1.107), h), ((-1.430, 0, 1.107), h)],
                        hmlt=hmlt)
    b.znuc, b.anuc = (8.0, 1.0, 1.0), (16.0, 1.0, 1.0)
    return b


@pytest.mark.parametrize("hmlt", ["DHFR", "DHFB"])
def test_scf_gpu_matches_oracle(hmlt):
    b = _water_small(hmlt)
    ref = DHFSCF(b, nocc=10, torch=torch,
                 backend=OracleBackend(b, breit=hmlt == "DHFB")).run(max_iter=40, etol=1e-10)
    assert ref["converged"]
    for prec, tol in (("fp64", 1e-9), ("df32", 1e-8)):
        scf = DHFSCF(b, nocc=10, precision=prec, screen=0.0)
        r = scf.run(max_iter=40, etol=1e-10)
        scf.close()
        assert r["converged"]
        assert abs(r["energy"] - ref["energy"]) < tol, (prec, r["energy"], ref["energy"])


def test_scf_atomic_guess_and_wfn_restart(tmp_path):
    """The superposed atomic start and a restart from the `.wfn` file the
    converged run wrote reach the bare-nucleus SCF's energy; the restart
    needs two iterations (the first already at the converged energy)."""
    from berthagpu import wfn
    b = _water_small()
    path = str(tmp_path / "water.wfn")
    s = DHFSCF(b, nocc=10, screen=0.0)
    r0 = s.run(max_iter=40, etol=1e-10, wfn_out=path)
    s.close()
    s = DHFSCF(b, nocc=10, screen=0.0)
    r1 = s.run(max_iter=40, etol=1e-10, guess="atomic")
    s.close()
    eign, coef = wfn.read_wfn(path, b.ndim)
    s = DHFSCF(b, nocc=10, screen=0.0)
    r2 = s.run(max_iter=40, etol=1e-10, guess=(eign, coef))
    s.close()
    assert r0["converged"] and r1["converged"] and r2["converged"]
    assert abs(r1["energy"] - r0["energy"]) < 1e-9
    assert abs(r2["energy"] - r0["energy"]) < 1e-9
    assert r2["iterations"] <= 3

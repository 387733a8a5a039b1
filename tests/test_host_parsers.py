"""Host-side readers of the C-ABI, run without a device: the FCIDUMP reader
(SHCI/integral.cpp:43-225) and the input reader for the variational keys
(SHCI/input.cpp:35-404), on the reference's own example inputs and on the
malformed inputs the reference rejects."""
import gzip
import os
import shutil

import numpy as np
import pytest

from dice_gb300 import engine as eng

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _unpack(tmp_path, name):
    out = tmp_path / (name + ".FCIDUMP")
    with gzip.open(os.path.join(GOLDEN, name + ".FCIDUMP.gz"), "rb") as f, open(out, "wb") as g:
        shutil.copyfileobj(f, g)
    return out


def _write(tmp_path, text, name="input.dat"):
    p = tmp_path / name
    p.write_text(text)
    return p


def test_fcidump_header_and_integrals_match_oracle(tmp_path):
    from oracle import oracle as orc
    orc.build()
    for name in ("h8_631g", "n2_RAS", "o2"):
        path = _unpack(tmp_path, name)
        n, ne, core, n2 = eng.fcidump_info(path)
        o = orc.Oracle(str(path))
        assert (n, ne) == (o.norb, o.nelec)
        assert core == o.coreE
        assert n2 == int(np.count_nonzero(o.i2()))


def test_fcidump_errors(tmp_path):
    with pytest.raises(eng.ShciError) as e:
        eng.fcidump_info(tmp_path / "missing")
    assert e.value.code == 2
    good = _unpack(tmp_path, "h8_631g").read_text().splitlines()
    end = next(i for i, l in enumerate(good) if "&END" in l.upper() or l.strip() == "/")
    # no end of the namelist header
    p = _write(tmp_path, "\n".join(good[:end]) + "\n", "noend")
    with pytest.raises(eng.ShciError) as e:
        eng.fcidump_info(p)
    assert e.value.code == 1
    # an orbital index beyond NORB
    bad = good[:end + 1] + ["0.5 17 1 1 1"] + good[end + 1:]
    p = _write(tmp_path, "\n".join(bad) + "\n", "range")
    with pytest.raises(eng.ShciError) as e:
        eng.fcidump_info(p)
    assert e.value.code == 1


def test_input_schedules_of_reference_examples(tmp_path):
    info = eng.input_info(os.path.join(GOLDEN, "h8_631g.dice.dat"))
    assert info["eps1"] == [1e-6] * 12
    assert info["nroots"] == 1 and info["ndet"] == 1 and info["nact"] == 8
    assert info["davidsonTol"] == 1e-8 and info["dE"] == 1e-10
    info = eng.input_info(os.path.join(GOLDEN, "n2_RAS.input.dat"))
    assert info["eps1"] == [1e-9] * 6
    info = eng.input_info(os.path.join(GOLDEN, "restart.input3.dat"))
    assert info["eps1"] == [5e-3] * 3 + [1e-3] * 3 + [5e-5] * 3
    assert info["davidsonTolLoose"] == 5e-5
    assert info["precision"] == -1 and info["precond"] == -1 and info["davidson_basis"] == 0


def test_input_engine_keywords(tmp_path):
    base = "nocc 2\n0 1\nend\nschedule\n0 1e-3\n2 1e-4\nend\nmaxiter 4\n"
    info = eng.input_info(_write(tmp_path, base + "precision mixed\nblockdavidson\nprecond mlp\n"
                                 "davidsonBasis 16 8\nnroots 3\n"))
    assert info["eps1"] == [1e-3, 1e-3, 1e-4, 1e-4]
    assert (info["precision"], info["blockdavidson"], info["precond"], info["davidson_basis"], info["nroots"]) == \
        (1, 1, 2, 16, 3)


@pytest.mark.parametrize("text,msg", [
    ("nocc 2\n0 1\nend\nschedule\n0 1e-3\nend\nmaxiter 4\nfrobnicate 3\n", "cannot read option"),
    ("nocc 2\n0 1\nend\nmaxiter 4\n", "schedule"),
    ("nocc 2\n0 1\nend\nschedule\n5 1e-3\nend\nmaxiter 4\n", "maxiter"),
    ("schedule\n0 1e-3\nend\nmaxiter 4\n", "nocc"),
    ("nocc 2\n0 1\nend\nschedule\n0 1e-3\nend\nmaxiter 4\nprecision half\n", "precision"),
    ("nocc 2\n0 1\nend\nschedule\n0 1e-3\nend\nmaxiter 4\ndavidsonBasis 32 8\n", "davidsonBasis"),
    ("nocc 2\n0 1\nend\nschedule\n0 1e-3\nend\nmaxiter 4\nTreversal 2\n", "Treversal"),
])
def test_input_errors(tmp_path, text, msg):
    """Malformed inputs and invalid values (a Treversal other than 0, 1 or -1,
    as SHCI/input.cpp:253-258 rejects) are rejected with SHCI_ERR_INVALID and
    the reason."""
    with pytest.raises(eng.ShciError) as e:
        eng.input_info(_write(tmp_path, text))
    assert e.value.code == 1
    assert msg in str(e.value)

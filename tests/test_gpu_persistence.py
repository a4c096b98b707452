"""Factor files (hodlr3d_save / hodlr3d_load): an operator saved after
assembly and loaded into a new handle gives bit-identical ranks, pivots and
products in every form, without running ACA; damaged files are refused with
HODLR3D_ERR_IO (a host-side check: nothing reaches the GPU)."""
import numpy as np
import pytest
import torch

from golden_util import golden_names, load, points_of

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=golden_names()[:3])
def saved(request, tmp_path_factory):
    from hodlr3d_gb300 import HODLR3D
    g = load(request.param)
    H = HODLR3D(int(g["nP1D"]), float(g["L"]), int(g["tol_pow"]), int(g["kernel"]), points_of(g),
                diag_override=float(g["diag"]))
    H.assemble()
    path = tmp_path_factory.mktemp("fact") / f"{request.param}.h3d"
    H.save(path)
    yield H, path
    H.close()


def test_load_reproduces_the_operator(saved):
    from hodlr3d_gb300 import HODLR3D
    H, path = saved
    G = HODLR3D.load(path)
    try:
        assert G.N == H.N and G.Qchoice == H.Qchoice and G.TOL_POW == H.TOL_POW
        assert np.array_equal(G.pairs(), H.pairs())
        assert np.array_equal(G.ranks(), H.ranks())
        for a, b in zip(G.pivots(), H.pivots()):
            assert np.array_equal(a, b)
        X = torch.tensor(np.random.default_rng(3).standard_normal((H.N, 3)), device="cuda")
        for prec in ("fp64", "mixed", "fp64x"):
            for tr in (False, True):
                assert torch.equal(G.matvec(X, prec, transpose=tr), H.matvec(X, prec, transpose=tr))
        assert G.stats()["aca_batches"] == 0  # no assembly ran
    finally:
        G.close()


def test_damaged_files_are_refused(saved, tmp_path):
    from hodlr3d_gb300 import HODLR3D, HODLR3DError
    from hodlr3d_gb300 import _lib
    H, path = saved
    data = bytearray(path.read_bytes())
    bad = tmp_path / "flipped.h3d"
    flipped = bytearray(data)
    flipped[len(flipped) - 100] ^= 0x40  # inside the last factor pool
    bad.write_bytes(bytes(flipped))
    with pytest.raises(HODLR3DError, match="checksum") as e:
        HODLR3D.load(bad)
    assert e.value.code == _lib.ERR_IO
    cut = tmp_path / "truncated.h3d"
    cut.write_bytes(bytes(data[: len(data) // 2]))
    with pytest.raises(HODLR3DError) as e:
        HODLR3D.load(cut)
    assert e.value.code == _lib.ERR_IO
    junk = tmp_path / "junk.h3d"
    junk.write_bytes(b"not a factor file" * 10)
    with pytest.raises(HODLR3DError) as e:
        HODLR3D.load(junk)
    assert e.value.code == _lib.ERR_IO
    with pytest.raises(HODLR3DError) as e:
        HODLR3D.load(tmp_path / "missing.h3d")
    assert e.value.code == _lib.ERR_IO

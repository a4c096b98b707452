"""Engine autotuning (hodlr3d_autotune).  On a 32^3 grid, where every engine
applies to A x, the tuner times each engine of the mixed product at 1, 2, 4,
8, 16, 32 and 64 columns, and the automatic choice then follows the fastest.
Checked: the timing table lists exactly the engines that apply (no
tensor-core transpose); the choice for each column count is a fastest engine
of the next timed count up; a product under the tuned automatic choice is
bit-identical to the same engine forced and within the mixed tolerance of the
FP64 form; reps=0 and a loaded operator use the column-count rules."""
import pytest
import torch

pytestmark = pytest.mark.gpu

COUNTS = (1, 2, 4, 8, 16, 32, 64)


@pytest.fixture(scope="module")
def tuned():
    from hodlr3d_gb300 import HODLR3D
    from hodlr3d_gb300.workloads import grid_cell_centres
    H = HODLR3D(4, 1.0, 10, 16, grid_cell_centres(32))
    H.assemble()
    rows = H.autotune(reps=3)
    yield H, rows
    H.close()


def test_table_lists_the_engines_that_apply(tuned):
    _, rows = tuned
    fwd = {(n, e) for t, n, e, _ in rows if not t}
    trn = {(n, e) for t, n, e, _ in rows if t}
    assert fwd == {(n, e) for n in COUNTS for e in ("simt", "tc", "gemv")}
    assert trn == {(n, e) for n in COUNTS for e in ("simt", "gemv")}
    assert all(ms > 0 for *_, ms in rows)


def test_choice_is_a_fastest_engine_of_the_next_timed_count(tuned):
    H, rows = tuned
    ms = {(t, n, e): v for t, n, e, v in rows}
    fastest = {}
    for (t, n, _), v in ms.items():
        fastest[(t, n)] = min(v, fastest.get((t, n), v))
    tun = H.tuning()
    for t, key in ((False, "forward"), (True, "transpose")):
        for n in range(1, 65):
            up = min(c for c in COUNTS if c >= n)
            assert ms[(t, up, tun[key][n - 1])] == fastest[(t, up)], (key, n)


@pytest.mark.parametrize("transpose", [False, True])
@pytest.mark.parametrize("nrhs", [1, 3, 8, 32, 40])
def test_tuned_product_equals_the_forced_engine(tuned, nrhs, transpose):
    H, _ = tuned
    eng = H.tuning()["transpose" if transpose else "forward"][nrhs - 1]
    g = torch.Generator(device="cpu").manual_seed(nrhs)
    X = torch.randn(H.N, nrhs, generator=g, dtype=torch.float64).cuda()
    y_auto = H.matvec(X, "mixed", transpose=transpose)
    H.set_engine(eng)
    try:
        y_forced = H.matvec(X, "mixed", transpose=transpose)
    finally:
        H.set_engine("auto")
    H.device_status()
    assert torch.equal(y_auto, y_forced)
    y64 = H.matvec(X, "fp64", transpose=transpose)
    err = (torch.linalg.norm(y_auto - y64, dim=0) / torch.linalg.norm(y64, dim=0)).max().item()
    assert err <= 2e-6


def test_reset_bad_reps_and_loaded_operators(tmp_path):
    from hodlr3d_gb300 import HODLR3D, HODLR3DError
    from hodlr3d_gb300.workloads import grid_cell_centres
    H = HODLR3D(4, 1.0, 10, 16, grid_cell_centres(16))
    H.assemble()
    with pytest.raises(HODLR3DError):
        H.autotune(reps=-1)
    rows = H.autotune(reps=1)
    assert len(rows) == 5 * len(COUNTS)
    t = H.tuning()
    assert None not in t["forward"] and None not in t["transpose"]
    assert "tc" not in t["transpose"]
    H.save(tmp_path / "op.h3d")
    G = HODLR3D.load(tmp_path / "op.h3d")
    assert set(G.tuning()["forward"] + G.tuning()["transpose"]) == {None}
    assert H.autotune(reps=0) == []
    assert set(H.tuning()["forward"] + H.tuning()["transpose"]) == {None}
    G.close()
    H.close()


def test_launch_shape_tuning(tuned):
    """The tuner also times the tensor-core T kernel at 1..32 blocks per slice
    (32 columns) and keeps the fastest; the product does not depend on it."""
    H, _ = tuned
    lt = H.launch_tuning()
    assert set(lt["ta_split"]) == {1, 2, 4, 8, 16, 32}
    assert all(v > 0 for v in lt["ta_split"].values())
    k = lt["ta_split_chosen"]
    assert lt["ta_split"][k] == min(lt["ta_split"].values())
    g = torch.Generator(device="cpu").manual_seed(7)
    X = torch.randn(H.N, 32, generator=g, dtype=torch.float64).cuda()
    H.set_engine("tc")
    try:
        y_tuned = H.matvec(X, "mixed")
        torch.cuda.synchronize()
        rows = H.autotune(reps=0)  # back to the default launch shapes
        assert rows == [] and H.launch_tuning()["ta_split_chosen"] is None
        y_rule = H.matvec(X, "mixed")
        torch.cuda.synchronize()
        assert torch.equal(y_tuned, y_rule)
    finally:
        H.set_engine("auto")
        H.autotune(reps=3)


def test_tuner_waits_for_products_in_flight(tuned):
    """A product queued on torch's stream, then the tuner (which runs its
    products on the handle's stream with the same work buffers) before any
    synchronisation: the queued product's result is still exact."""
    H, _ = tuned
    g = torch.Generator(device="cpu").manual_seed(8)
    X = torch.randn(H.N, 32, generator=g, dtype=torch.float64).cuda()
    H.set_engine("tc")
    try:
        ref = H.matvec(X, "mixed")
        torch.cuda.synchronize()
        y = H.matvec(X, "mixed")
        H.autotune(reps=1)  # no synchronisation before it
        torch.cuda.synchronize()
        assert torch.equal(y, ref)
    finally:
        H.set_engine("auto")
        H.autotune(reps=3)

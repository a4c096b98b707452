"""The bounded waits of the tensor-core engine, run out on purpose without a
GPU fault.  hodlr3d_test_drop_copy makes block (0, 0) of the T kernel stop
copying before a chunk, so the "landed" barrier of that chunk is never
completed (a flag that nothing sets).  The block's waits give up after about
a second, it drains the copies and products it has in flight and frees its
tensor memory, hodlr3d_device_status reports the failure once, and the next
product on the same handle is bit-identical to the one before the failure
(the context stays usable)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_tensor_core_wait_gives_up_and_handle_recovers():
    from hodlr3d_gb300 import HODLR3D
    from hodlr3d_gb300._lib import ERR_CUDA, HODLR3DError, check
    from hodlr3d_gb300.workloads import grid_cell_centres
    # 32^3: depth 3, so the T kernel has work (level-2 pairs)
    H = HODLR3D(4, 1.0, 10, 16, grid_cell_centres(32))
    H.assemble()
    try:
        X = torch.tensor(np.random.default_rng(4).standard_normal((H.N, 32)), device="cuda")
        H.set_engine("tc")
        y0 = H.matvec(X, "mixed")
        H.device_status()
        for chunk in (0, 3):
            check(H._L.hodlr3d_test_drop_copy(H.handle, chunk))
            H.matvec(X, "mixed")
            with pytest.raises(HODLR3DError, match="gave up") as e:
                H.device_status()
            assert e.value.code == ERR_CUDA
            H.device_status()  # reported once
            y1 = H.matvec(X, "mixed")
            H.device_status()
            assert torch.equal(y1, y0)
        with pytest.raises(HODLR3DError):
            check(H._L.hodlr3d_test_drop_copy(H.handle, -2))
    finally:
        H.set_engine("auto")
        H.close()

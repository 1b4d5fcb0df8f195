"""tea_gb300_dot_noalloc: the dot product for callers that cannot allocate.

Some hosts cannot call cudaMalloc on the path that needs a reduction:
their GPU memory belongs to another allocator, or allocation is not allowed
there.  tea_gb300_dot_noalloc takes caller-owned inputs and output and keeps
its scratch in a fixed device array inside the library.  This test checks,
through the C ABI, that it returns the same bits as the library's existing
2-norm entry point on the same data, on two calls in a row, and that an
interior too large for its fixed scratch is refused.

The file name sorts last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def device_copy(torch, arr):
    return torch.from_numpy(np.ascontiguousarray(arr)).to("cuda")


def test_dot_noalloc_matches_calc_2norm_twice():
    torch = pytest.importorskip("torch")
    from tealeaf_opencl_gb300 import decks, lib
    L = lib.load()
    x, y, H = 300, 67, 2
    ch = lib.Chunk(x, y, H, "cg", "jac_diag")
    ch.set_arithmetic(True)
    decks.setup_five_state(ch, x, y)
    ch.common_init(1, 0.004)
    ch.calc_residual()
    expected = [ch.calc_2norm(1), ch.calc_2norm(0)]   # r.r, u0.u0
    fields = [ch.read_padded("r"), ch.read_padded("u0")]

    stride = x + 2 * H
    result = torch.zeros(1, dtype=torch.float64, device="cuda")
    got = []
    for f in fields:
        a = device_copy(torch, f)
        rc = L.tea_gb300_dot_noalloc(a.data_ptr(), a.data_ptr(), x, y, H, stride,
                                     result.data_ptr(), None)
        assert rc == 0, lib.check()
        torch.cuda.synchronize()
        got.append(float(result.cpu()[0]))
    assert got == expected


@pytest.mark.parametrize("fused", [True, False], ids=["fused", "exact"])
def test_dot_noalloc_two_fields_and_tall_tiles(fused):
    """r.z on a grid with 16-row reduction tiles, in both arithmetic forms."""
    torch = pytest.importorskip("torch")
    from tealeaf_opencl_gb300 import lib
    L = lib.load()
    x, y, H = 2048, 2440, 1
    assert L.tea_gb300_reduction_rows(x, y) == 16
    ch = lib.Chunk(x, y, H, "cg", "jac_diag")   # with a preconditioner, 2norm(2) is r.z
    ch.set_arithmetic(fused)
    rng = np.random.default_rng(4)
    ch.write("r", rng.standard_normal((y, x)))
    ch.write("z", rng.standard_normal((y, x)))
    expected = ch.calc_2norm(2)
    a = device_copy(torch, ch.read_padded("r"))
    b = device_copy(torch, ch.read_padded("z"))
    result = torch.zeros(1, dtype=torch.float64, device="cuda")
    for _ in range(2):
        result.zero_()
        rc = L.tea_gb300_dot_noalloc(a.data_ptr(), b.data_ptr(), x, y, H,
                                     x + 2 * H, result.data_ptr(), None)
        assert rc == 0
        torch.cuda.synchronize()
        assert float(result.cpu()[0]) == expected


def test_dot_noalloc_rejects_interior_beyond_scratch():
    from tealeaf_opencl_gb300 import lib
    L = lib.load()
    buf = ctypes.c_double(0.0)
    p = ctypes.addressof(buf)
    # the bound is on supertiles (8 x 32 columns by 16 rows here), not on
    # the side length: a wide square and a thin, tall strip both exceed it
    for x, y in ((20000, 20000), (32, 2_200_000)):
        rc = L.tea_gb300_dot_noalloc(p, p, x, y, 1, x + 2, p, None)
        assert rc == -1
        msg = ctypes.create_string_buffer(512)
        assert L.tea_gb300_last_error(msg, 512) != 0
        assert b"partial sums of the fixed scratch" in msg.value

"""gf_plaquette_noalloc: the plaquette sum for callers that cannot allocate
device memory (their device memory belongs to another allocator, such as
CUDA.jl's pool or PyTorch's caching allocator, or they run a loop where a
cudaMalloc would synchronise the device). It keeps its partial sums in a
fixed device array inside the library instead of a context's buffer.

Called through the C-ABI and checked against gf_plaquette, the entry point
with a context, within the plaquette tolerance of the parity tests (1e-13
relative), on two calls in a row (the shared array keeps the previous call's
contents, which must not leak into the next result). This file is collected
last so that a run stopping at the first failure has run every other test.
"""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def _call(lib, U, L, out, stream):
    Larr = (ctypes.c_int * 4)(*L)
    return lib.gf_plaquette_noalloc(ctypes.c_void_p(U.field.device_ptr()), Larr, ctypes.c_void_p(out),
                                    ctypes.c_void_p(stream))


def test_noalloc_plaquette_matches_gf_plaquette(pkg):
    import torch
    from gaugefields_gb300 import _lib
    lib = _lib.load()
    stream = torch.cuda.current_stream()
    for L, seed in (((8, 8, 8, 8), 1234), ((4, 6, 4, 8), 5), ((16, 16, 16, 16), 9)):
        U = pkg.gauge_configuration(L, start="hot", seed=seed)
        ref = pkg.calculate_Plaquette(U)  # synchronises the context's stream
        out = torch.full((2,), -1.0, dtype=torch.float64, device="cuda")
        for k in range(2):
            rc = _call(lib, U, L, out.data_ptr() + 8 * k, stream.cuda_stream)
            assert rc == 0, lib.gf_last_error(None)
        torch.cuda.synchronize()
        for k in range(2):
            got = out[k].item()
            assert abs(got - ref) <= 1e-13 * abs(ref), (L, k, got, ref)


def test_noalloc_plaquette_cold_start_is_exact(pkg):
    import torch
    from gaugefields_gb300 import _lib
    lib = _lib.load()
    L = (8, 8, 8, 8)
    U = pkg.gauge_configuration(L, start="cold")
    U.ctx.sync()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    assert _call(lib, U, L, out.data_ptr(), 0) == 0
    torch.cuda.synchronize()
    assert out.item() / (6 * 8 ** 4 * 3) == 1.0


def test_noalloc_plaquette_rejects_oversized_lattices(pkg):
    from gaugefields_gb300 import _lib
    lib = _lib.load()
    U = pkg.gauge_configuration((4, 4, 4, 4), start="cold")
    L = (256, 256, 256, 2)  # 2^25 sites: beyond the 2^24 the fixed array holds
    assert _call(lib, U, L, 0x1000, 0) == _lib.GF_EINVAL
    assert b"at most 16777216" in lib.gf_last_error(None)
    assert _call(lib, U, (3, 4, 4, 4), 0x1000, 0) == _lib.GF_EINVAL
    # extents whose product overflows 64 bits are rejected, not wrapped
    big = 1 << 16
    assert _call(lib, U, (big, big, big, big), 0x1000, 0) == _lib.GF_EINVAL
    assert _call(lib, U, (2, 2, 2, (1 << 30)), 0x1000, 0) == _lib.GF_EINVAL


def test_noalloc_plaquette_leaves_device_memory_untouched(pkg):
    """After the first call (which looks up the array's address), further
    calls change neither the device's free memory nor PyTorch's allocator."""
    import torch
    from gaugefields_gb300 import _lib
    lib = _lib.load()
    L = (8, 8, 8, 8)
    U = pkg.gauge_configuration(L, start="hot", seed=3)
    U.ctx.sync()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    assert _call(lib, U, L, out.data_ptr(), stream) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    alloc0, reserved0 = torch.cuda.memory_allocated(), torch.cuda.memory_reserved()
    for _ in range(20):
        assert _call(lib, U, L, out.data_ptr(), stream) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.cuda.memory_allocated() == alloc0 and torch.cuda.memory_reserved() == reserved0

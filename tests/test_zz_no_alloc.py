"""faces_share_static: the entry point for callers that cannot allocate.

Applications that give all device memory to their own pool, or loops that
cannot take the synchronisation cudaMalloc implies, call faces_share_static:
it keeps the message-mode working memory in a fixed device array inside the
library instead of allocating.  These tests call it through the C ABI and
check, over two calls in a row, that it gives exactly what faces_share with
FACES_MESSAGES gives (bit for bit, the tolerance of every parity test here),
and that a field too large for the array is refused with a clear error.
"""
import ctypes

import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)


def static_share(F):
    L = F.lib()
    fn = L.faces_share_static
    fn.argtypes = [ctypes.c_void_p] + [ctypes.c_int] * 7 + [ctypes.c_uint, ctypes.c_int, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


CASES = [
    # lx ly lz mx my mz n periodic
    (3, 3, 3, 2, 2, 2, 6, True),
    (2, 1, 1, 3, 2, 2, 5, False),
    (1, 1, 1, 4, 4, 4, 5, True),
    (2, 2, 1, 3, 1, 2, 8, True),
    (1, 2, 2, 2, 3, 2, 14, False),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "x".join(map(str, c[:7])) + ("p" if c[7] else "o"))
@pytest.mark.parametrize("compute", [True, False])
def test_static_share_matches_message_mode(faces_lib, case, compute):
    F = faces_lib
    fn = static_share(F)
    *shape, periodic = case
    ref = F.Faces(*shape, periodic=periodic, messages=True)
    a = ref.field()
    ref.init_ref(a)
    b = a.clone()
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        ref.share(a, compute, stream)
        rc = fn(b.data_ptr(), *shape, F.PERIODIC if periodic else 0, int(compute), stream)
        assert rc == 0, F.lib().faces_last_error().decode()
        torch.cuda.synchronize()
        assert torch.equal(a, b), f"call {call + 1}: {int((a != b).sum())} points differ"
    ref.close()


def test_static_share_refuses_oversized_field(faces_lib):
    F = faces_lib
    fn = static_share(F)
    u = torch.zeros(1024, dtype=torch.float64, device="cuda")
    rc = fn(u.data_ptr(), 6, 6, 6, 40, 40, 40, 8, F.PERIODIC, 1, None)
    assert rc == -1
    msg = F.lib().faces_last_error().decode()
    assert "static scratch holds" in msg and "faces_share with FACES_MESSAGES" in msg
    torch.cuda.synchronize()
    assert torch.count_nonzero(u) == 0  # nothing ran


def test_static_share_allocates_nothing(faces_lib):
    """After a first call of a shape (which loads the kernels it uses, and
    with them the module's device array, under lazy module loading), further
    calls leave the device's free memory (cudaMemGetInfo) and torch's
    allocator counters unchanged: nothing is allocated or freed."""
    F = faces_lib
    fn = static_share(F)
    shape = (3, 3, 3, 4, 4, 4, 6)
    f = F.Faces(*shape, periodic=True, messages=True)
    u = f.field()
    f.init_int(u, 3)
    stream = torch.cuda.current_stream().cuda_stream
    assert fn(u.data_ptr(), *shape, F.PERIODIC, 1, stream) == 0, F.lib().faces_last_error().decode()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    stats0 = torch.cuda.memory_stats()
    for _ in range(3):
        assert fn(u.data_ptr(), *shape, F.PERIODIC, 1, stream) == 0, F.lib().faces_last_error().decode()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    stats1 = torch.cuda.memory_stats()
    assert free1 == free0, f"free device memory changed by {free1 - free0} bytes"
    for key in ("allocation.all.allocated", "segment.all.allocated", "num_device_alloc"):
        assert stats1.get(key, 0) == stats0.get(key, 0), key
    # and the result is still the message-mode result of 4 shares
    chk = f.check(u, init="int", seed=3, nshares=4)
    assert chk.passed and chk.maxrel == 0.0, chk
    f.close()

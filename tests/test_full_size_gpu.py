"""The benchmark shapes at full size, bit for bit against the CPU oracle,
and the device check shown able to fail.

The bench reports its numbers on these fields, so they are pinned to the
oracle's own result at their full size (not only through the device closed
form): the 48^3 n=8 periodic field (one rank, direct and v-26 message mode),
the 3x3x3-rank grid of 16^3 n=6 elements (v-26 messages, v-6 and direct), and
the reference's own open 15x14x13 n=12 shape (gpu/frontier-run-all-1.sh:15).
On integer-valued inputs every summation order is exact, so any correct
formulation of the oracle gives the same bits; v-6 runs are compared with the
oracle's own v-6 restatement as well.

faces_check is the rule of gpu/main.cc:39-105 evaluated on the device against
a closed form.  Every large-shape test here and the bench's `check` rely on
it, so the last tests plant errors -- in a field point, in a padding double,
a NaN -- and require it to report each one, with the rank and place.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)


def run(F, shape, nshares, *, periodic=True, init="int", seed=11, autotune=False, tune=None, **mode):
    f = F.Faces(*shape, periodic=periodic, **mode)
    if tune:
        f.set_tuning(**tune)
    u = f.field()
    if init == "int":
        f.init_int(u, seed)
    else:
        f.init_ref(u)
    if autotune:
        f.autotune(u, True, 2)
        if init == "int":
            f.init_int(u, seed)
        else:
            f.init_ref(u)
    f.share_n(u, nshares)
    torch.cuda.synchronize()
    out = u.cpu().numpy()
    chk = f.check(u, init=init, seed=seed, nshares=nshares)
    f.close()
    return out, chk


def expected(O, shape, nshares, *, periodic=True, init="int", seed=11, v6=False):
    s = O.Shape(*shape, periodic=periodic)
    u = O.init_int(s, seed) if init == "int" else O.init_ref(s)
    return (O.v6_share if v6 else O.groups_share)(s, u, True, nshares)


C2 = (1, 1, 1, 48, 48, 48, 8)
C3 = (3, 3, 3, 16, 16, 16, 6)


@pytest.mark.parametrize("mode", ["direct", "direct-autotuned", "messages"])
def test_c2_full_size_equals_oracle(oracle, faces_lib, mode):
    """48^3 elements of n=8, periodic, 3 shares: 56.6 M points, bit for bit."""
    exp = expected(oracle, C2, 3)
    out, chk = run(faces_lib, C2, 3, messages=mode == "messages", autotune=mode == "direct-autotuned")
    assert np.array_equal(out, exp), f"{np.count_nonzero(out != exp)} points differ"
    assert chk.passed and chk.maxrel == 0.0


@pytest.mark.parametrize("mode", ["messages", "v6", "v6f", "direct"])
def test_c3_full_size_equals_oracle(oracle, faces_lib, mode):
    """3x3x3 periodic virtual ranks of 16^3 elements, n=6, 3 shares."""
    exp = expected(oracle, C3, 3, v6=mode.startswith("v6"))
    out, chk = run(faces_lib, C3, 3, messages=mode == "messages", v6=mode == "v6", v6f=mode == "v6f")
    assert np.array_equal(out, exp), f"{np.count_nonzero(out != exp)} points differ"
    assert chk.passed and chk.npass == 27
    if mode.startswith("v6"):
        assert np.array_equal(out, expected(oracle, C3, 3)), "v-6 differs from the group sums"


@pytest.mark.parametrize("mode", ["direct", "seams-lean", "general", "messages", "v6", "v6f"])
def test_reference_shape_open_equals_oracle(oracle, faces_lib, mode):
    """The reference's own argument set 1 1 1 15 14 13 12 (open, reference
    init, 2 shares): the same tree order as Mugs, so equal on any input.
    direct: the default (the seam kernel's chunked form at this size);
    seams-lean: its lean form; general: the general tile step."""
    shape = (1, 1, 1, 15, 14, 13, 12)
    exp = expected(oracle, shape, 2, periodic=False, init="ref", v6=mode.startswith("v6"))
    out, chk = run(faces_lib, shape, 2, periodic=False, init="ref", messages=mode == "messages", v6=mode == "v6",
                   v6f=mode == "v6f", general=mode == "general", seams=mode == "seams-lean",
                   tune={"order": 1} if mode == "seams-lean" else None)
    assert np.array_equal(out, exp), f"{np.count_nonzero(out != exp)} points differ"
    assert chk.passed


@pytest.mark.parametrize("periodic", [False, True], ids=["open", "periodic"])
def test_reference_large_shape_seams_equal_tiles(faces_lib, periodic):
    """The reference's 1 1 1 95 94 93 12 shape (1.4 G points) at full size,
    2 shares: the default (the seam kernel's lean form) equals the general
    tile step bit for bit on the device, and the device check passes."""
    F = faces_lib
    shape = (1, 1, 1, 95, 94, 93, 12)
    outs = []
    for general in (False, True):
        f = F.Faces(*shape, periodic=periodic, general=general)
        assert (f.tuning()["kernel"] == 3) != general
        u = f.field()
        f.init_ref(u)
        f.share_n(u, 2)
        chk = f.check(u, init="ref", nshares=2)
        assert chk.passed and chk.npass == 1, (general, chk)
        outs.append(u)
        f.close()
    assert torch.equal(outs[0], outs[1])


# -- faces_check must fail where the field is wrong --------------------------

NEG = (2, 1, 1, 3, 2, 2, 5)  # 2 ranks; jz slabs of 750 points padded to 1024


def _field(F):
    f = F.Faces(*NEG, periodic=True)
    u = f.field()
    f.init_int(u, 4)
    f.share_n(u, 2)
    torch.cuda.synchronize()
    assert f.check(u, init="int", seed=4, nshares=2).passed
    return f, u


@pytest.mark.parametrize("where", [(1, 0, 2, 4, 1, 1, 0), (0, 2, 2, 2, 2, 0, 1), (1, 4, 4, 4, 2, 1, 1)],
                         ids=["seam", "interior", "corner"])
def test_check_reports_a_wrong_point(faces_lib, where):
    f, u = _field(faces_lib)
    r, ix, iy, iz, jx, jy, jz = where
    i = f.index(ix, iy, iz, jx, jy, jz, rank=r)
    good = float(u[i])
    u[i] = good + 1.0
    chk = f.check(u, init="int", seed=4, nshares=2)
    assert not chk.passed and chk.npass == f.nranks - 1
    assert chk.where == where
    assert chk.values == (good + 1.0, good)
    assert chk.rank_maxrel[1 - r] == 0.0 and chk.rank_maxrel[r] > 1e-15
    f.close()


def test_check_reports_a_padding_write(faces_lib):
    f, u = _field(faces_lib)
    n, mx, my = 5, 3, 2
    plane = n ** 3 * mx * my
    i = 1 * f.rank_doubles + 1 * f.strides[5] + plane + 17  # rank 1, jz = 1, padding double 17
    u[i] = 3.0
    chk = f.check(u, init="int", seed=4, nshares=2)
    assert not chk.passed and chk.npass == f.nranks - 1
    assert chk.maxrel == 1.0
    assert chk.where == (1, -1, -1, -1, -1, -1, 1)
    assert chk.values == (3.0, 0.0)
    f.close()


def test_check_reports_nan(faces_lib):
    f, u = _field(faces_lib)
    u[f.index(1, 1, 0, 2, 1, 0, rank=0)] = float("nan")
    chk = f.check(u, init="int", seed=4, nshares=2)
    assert not chk.passed and chk.npass == f.nranks - 1
    assert chk.maxrel == float("inf")
    assert chk.where == (0, 1, 1, 0, 2, 1, 0)
    f.close()


def test_check_reports_a_wrong_share_count(faces_lib):
    """A field one share behind fails on every rank."""
    f, u = _field(faces_lib)
    chk = f.check(u, init="int", seed=4, nshares=3)
    assert not chk.passed and chk.npass == 0
    f.close()

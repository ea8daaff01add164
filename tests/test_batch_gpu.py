"""Batches: many fields of different shapes advanced by one persistent launch
per share must give every field exactly what faces_share gives it alone,
and what the oracle gives."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)


# lx ly lz mx my mz n, periodic, messages
MIX = [
    ((1, 1, 1, 4, 4, 4, 5), False, False),
    ((1, 1, 1, 3, 2, 5, 8), True, False),
    ((1, 1, 1, 1, 1, 1, 3), False, False),
    ((2, 1, 1, 3, 2, 2, 4), True, False),
    ((1, 2, 2, 2, 3, 2, 6), False, False),
    ((3, 3, 3, 2, 2, 2, 6), True, False),
    ((2, 2, 2, 1, 1, 1, 7), False, False),
    ((1, 1, 1, 5, 2, 3, 10), True, False),
    ((1, 1, 1, 9, 2, 2, 2), False, False),
    ((1, 3, 1, 3, 1, 2, 9), True, False),
    ((2, 1, 2, 2, 2, 1, 12), False, False),   # n > 10: one faces_share of its own
    ((2, 1, 1, 3, 2, 2, 5), True, True),      # messages: one faces_share of its own
    ((1, 1, 1, 17, 3, 2, 8), False, False),
]


def make_fields(F, mix, seed0=11):
    out = []
    for i, (shape, periodic, messages) in enumerate(mix):
        f = F.Faces(*shape, periodic=periodic, messages=messages)
        u = f.field()
        f.init_int(u, seed0 + i)
        out.append((f, u))
    return out


def alone(F, mix, nshares, compute=True, seed0=11):
    res = []
    for f, u in make_fields(F, mix, seed0):
        f.share_n(u, nshares, compute)
        torch.cuda.synchronize()
        res.append(u.cpu().numpy())
        f.close()
    return res


def batched(F, mix, nshares, how, compute=True, seed0=11, tune=None):
    fields = make_fields(F, mix, seed0)
    b = F.Batch()
    for f, u in fields:
        b.add(f, u)
    b.commit()
    if tune:
        b.tune(*tune)
    if how == "share":
        for _ in range(nshares):
            b.share(compute)
    elif how == "graph":
        b.share_n(nshares, compute)
    else:
        for _ in range(nshares):
            b.share_each(compute)
    torch.cuda.synchronize()
    info = b.info()
    b.close()
    res = [u.cpu().numpy() for _, u in fields]
    for f, _ in fields:
        f.close()
    return res, info


@pytest.mark.parametrize("how", ["share", "graph", "each"])
@pytest.mark.parametrize("compute", [True, False], ids=["compute", "nocompute"])
def test_batch_equals_alone(faces_lib, how, compute):
    F = faces_lib
    ref = alone(F, MIX, 3, compute)
    got, info = batched(F, MIX, 3, how, compute)
    assert info["fields"] == len(MIX)
    assert info["fused_fields"] == len(MIX) - 2
    for i, (a, b) in enumerate(zip(ref, got)):
        assert np.array_equal(a, b), f"field {i} {MIX[i]}"


@pytest.mark.parametrize("tune", [(1, 1), (2, 2, -1, 3), (4, 3), (8, 0, -1, 1), (64, 1, -1, 8)], ids=str)
def test_batch_work_split(faces_lib, tune):
    F = faces_lib
    ref = alone(F, MIX, 2)
    got, info = batched(F, MIX, 2, "share", tune=tune)
    assert info["unit_div"] == tune[0]
    for i, (a, b) in enumerate(zip(ref, got)):
        assert np.array_equal(a, b), f"field {i} {MIX[i]}"


def test_batch_matches_oracle(oracle, faces_lib):
    O, F = oracle, faces_lib
    mix = MIX[:6]
    got, _ = batched(F, mix, 2, "graph", seed0=3)
    for i, ((shape, periodic, messages), out) in enumerate(zip(mix, got)):
        s = O.Shape(*shape, periodic=periodic)
        u = O.init_int(s, 3 + i)
        for _ in range(2):
            O.groups_share(s, u)
        assert np.array_equal(u, out), f"field {i} {shape}"


def test_graph_replay_and_autotune(faces_lib):
    """A captured graph replays on later calls; autotune keeps results exact."""
    F = faces_lib
    mix = [((1, 1, 1, 6, 5, 4, n), n % 2 == 0, False) for n in range(2, 11)]
    fields = make_fields(F, mix, 40)
    b = F.Batch()
    for f, u in fields:
        b.add(f, u)
    b.commit()
    applied = b.autotune(trials=1)
    assert applied >= 8
    for _ in range(3):
        b.share_n(2)
    torch.cuda.synchronize()
    got = [u.cpu().numpy() for _, u in fields]
    info = b.info()
    b.close()
    for f, _ in fields:
        f.close()
    ref = alone(F, mix, 6 + applied, seed0=40)
    for i, (a, c) in enumerate(zip(ref, got)):
        assert np.array_equal(a, c), f"field {i} {mix[i]} {info}"


def test_many_fields(faces_lib):
    """512 small fields of uneven shape in one launch."""
    F = faces_lib
    rng = np.random.default_rng(7)
    mix = []
    for _ in range(512):
        n = int(rng.integers(2, 11))
        m = tuple(int(x) for x in rng.integers(1, 5, size=3))
        mix.append(((1, 1, 1) + m + (n,), bool(rng.integers(0, 2)), False))
    ref = alone(F, mix, 2, seed0=100)
    got, info = batched(F, mix, 2, "graph", seed0=100)
    assert info["fused_fields"] == 512
    bad = [i for i, (a, b) in enumerate(zip(ref, got)) if not np.array_equal(a, b)]
    assert not bad, [mix[i] for i in bad[:5]]


@pytest.mark.parametrize("half", [0, 1], ids=["full_tiles", "half_tiles"])
def test_all_periodic_batch_equals_general_step(faces_lib, half):
    """A batch of periodic direct-mode fields runs the periodic tile step
    only (full or half-length tiles); it must equal the general tile step of
    each field alone."""
    F = faces_lib
    rng = np.random.default_rng(11)
    mix = []
    for _ in range(40):
        L = tuple(int(x) for x in rng.integers(1, 3, size=3))
        m = tuple(int(x) for x in rng.integers(1, 9, size=3))
        mix.append((L + m + (int(rng.integers(2, 11)),), True, False))
    got, info = batched(F, mix, 3, "graph", seed0=500, tune=(0, 0, half))
    assert info["fused_fields"] == len(mix) and info["half"] == half
    for i, ((shape, _, _), out) in enumerate(zip(mix, got)):
        f = F.Faces(*shape, periodic=True, general=True)
        u = f.field()
        f.init_int(u, 500 + i)
        f.share_n(u, 3)
        torch.cuda.synchronize()
        assert np.array_equal(u.cpu().numpy(), out), f"field {i} {shape}"
        f.close()


def test_half_tiles_need_periodic_fields(faces_lib):
    F = faces_lib
    fields = make_fields(F, MIX[:4], 1)
    b = F.Batch()
    for f, u in fields:
        b.add(f, u)
    b.commit()
    with pytest.raises(F.FacesError):
        b.tune(0, 0, 1)
    b.close()
    for f, _ in fields:
        f.close()


# periodic fields only (the warp form needs every batched field on the
# periodic step): small n for the warp form, larger n for the block pipeline
WARP_MIX = [((1, 1, 1, m[0], m[1], m[2], n), True, False) for m, n in (
    ((3, 2, 4), 2), ((5, 3, 2), 3), ((24, 2, 3), 3), ((1, 1, 1), 3), ((7, 4, 4), 4), ((11, 2, 5), 4),
    ((13, 3, 2), 5), ((6, 6, 6), 5), ((2, 9, 2), 5), ((4, 3, 5), 6), ((9, 2, 2), 7), ((3, 4, 3), 8),
    ((2, 2, 7), 10))] + [((2, 1, 2, 3, 2, 2, 4), True, False), ((1, 2, 1, 7, 2, 3, 5), True, False)]


@pytest.mark.parametrize("warp", [(0, 1), (3, 1), (5, 2), (5, 4), (4, 3)], ids=lambda w: f"max_n{w[0]}-boost{w[1]}")
@pytest.mark.parametrize("half", [0, 2])
def test_warp_form_equals_alone(oracle, faces_lib, warp, half):
    """Small-n fields taken warp by warp in the same launch as the block
    pipeline: every field as alone and as the oracle gives it, bit for bit."""
    O, F = oracle, faces_lib
    exp = alone(F, WARP_MIX, 3)
    fields = make_fields(F, WARP_MIX)
    b = F.Batch()
    for f, u in fields:
        b.add(f, u)
    b.commit()
    b.tune(0, 0, half, 0)
    b.tune_warp(*warp)
    info = b.info()
    assert info["warp_max_n"] == warp[0]
    assert (info["warp_units"] > 0) == (warp[0] >= 2)
    b.share_n(3)
    torch.cuda.synchronize()
    for i, ((f, u), e) in enumerate(zip(fields, exp)):
        assert np.array_equal(u.cpu().numpy(), e), f"field {i} {WARP_MIX[i][0]}"
    sh = WARP_MIX[6][0]
    s = O.Shape(*sh, periodic=True)
    assert np.array_equal(fields[6][1].cpu().numpy(), O.groups_share(s, O.init_int(s, 17), True, 3))
    b.close()
    for f, _ in fields:
        f.close()


def test_v6_members_keep_their_order(faces_lib):
    """v-6 fields sum in the order z, y, x; in a batch they run alone (one
    faces_share each), so on the reference's non-integer init they still
    give exactly their alone result, beside fields the batched kernel takes."""
    F = faces_lib
    specs = [((1, 1, 1, 3, 2, 4, 5), dict(periodic=True, v6=True)), ((2, 1, 1, 2, 3, 2, 6), dict(v6f=True)),
             ((1, 1, 1, 4, 3, 2, 5), dict(periodic=True)), ((1, 2, 1, 3, 2, 2, 8), dict(periodic=True, v6f=True))]
    def fields():
        out = []
        for sh, kw in specs:
            f = F.Faces(*sh, **kw)
            u = f.field()
            f.init_ref(u)
            out.append((f, u))
        return out
    exp = []
    for f, u in fields():
        f.share_n(u, 3)
        torch.cuda.synchronize()
        exp.append(u.cpu().numpy())
        f.close()
    got = fields()
    b = F.Batch()
    for f, u in got:
        b.add(f, u)
    b.commit()
    assert b.info()["fused_fields"] == 1
    b.share_n(3)
    torch.cuda.synchronize()
    for i, ((f, u), e) in enumerate(zip(got, exp)):
        assert np.array_equal(u.cpu().numpy(), e), f"field {i}"
        f.close()
    b.close()

"""GPU parity: the sm_103a kernels against the CPU oracle, bit for bit.

Every kernel forms each shared point's sum as the tree x pairs -> y pairs ->
z pairs, the order of the reference's Mugs passes (gpu/Mugs.cc:140-202), so
the comparison is exact for any input -- integer-valued (where every order is
exact) and the reference's non-integer init (gpu/main.cc:18) alike.
"""
import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)


def run_gpu(F, s, *, periodic, messages, gather=False, rows=False, general=False, init="int", seed=5, nsteps=2,
            compute=True, seams=False, tune=None):
    f = F.Faces(s.lx, s.ly, s.lz, s.mx, s.my, s.mz, s.n, periodic=periodic, messages=messages, gather=gather,
                rows=rows, general=general, seams=seams)
    if tune:
        f.set_tuning(**tune)
    u = f.field()
    if init == "int":
        f.init_int(u, seed)
    else:
        f.init_ref(u)
    u_init = u.cpu().numpy()
    f.share_n(u, nsteps, compute)
    torch.cuda.synchronize()
    out = u.cpu().numpy()
    chk = f.check(u, init=init, seed=seed, nshares=nsteps, compute=compute)
    f.close()
    return u_init, out, chk


SHAPES = [
    # lx ly lz mx my mz n
    (1, 1, 1, 4, 4, 4, 5),      # the C1 shape
    (1, 1, 1, 3, 2, 5, 8),
    (1, 1, 1, 1, 1, 1, 3),
    (1, 1, 1, 2, 3, 1, 2),
    (2, 1, 1, 3, 2, 2, 4),
    (1, 2, 2, 2, 3, 2, 6),
    (3, 3, 3, 2, 2, 2, 6),      # the C3 rank grid, small elements
    (2, 2, 2, 1, 1, 1, 7),
    (1, 1, 1, 5, 2, 3, 10),
    (2, 1, 2, 2, 2, 1, 12),
    (1, 1, 1, 2, 2, 2, 16),
    (1, 3, 1, 3, 1, 2, 9),
]


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
@pytest.mark.parametrize("periodic", [False, True], ids=["open", "periodic"])
@pytest.mark.parametrize("messages", [False, True], ids=["direct", "messages"])
@pytest.mark.parametrize("kernel", ["tiles", "general", "rows", "seams", "seams-lean"])
def test_step_bit_exact(oracle, faces_lib, shape, periodic, messages, kernel):
    """tiles: the periodic tile step where it applies (periodic direct mode),
    else the general one; general: the general tile step everywhere; seams:
    the seam kernel (direct mode only), one launch or split in two."""
    O, F = oracle, faces_lib
    if kernel == "general" and not (periodic and not messages):
        pytest.skip("same kernel as 'tiles' here")
    if kernel.startswith("seams") and messages:
        pytest.skip("the seam kernel sums in place (direct mode)")
    s = O.Shape(*shape, periodic=periodic)
    for init in ("int", "ref"):
        u_init, out, chk = run_gpu(F, s, periodic=periodic, messages=messages, rows=kernel == "rows",
                                   general=kernel == "general", init=init, nsteps=3, seams=kernel.startswith("seams"),
                                   tune={"order": 1} if kernel == "seams-lean" else None)
        ref0 = O.init_int(s, 5) if init == "int" else O.init_ref(s)
        assert np.array_equal(u_init, ref0), "device init differs from the host formula"
        exp = O.groups_share(s, ref0.copy(), True, 3)
        assert np.array_equal(out, exp), f"{init}: {np.count_nonzero(out != exp)} points differ"
        assert chk.passed and chk.npass == s.nranks


@pytest.mark.parametrize("shape", SHAPES[:8], ids=lambda s: "x".join(map(str, s)))
@pytest.mark.parametrize("periodic", [False, True], ids=["open", "periodic"])
@pytest.mark.parametrize("messages", [False, True], ids=["direct", "messages"])
def test_without_compute_kernels(oracle, faces_lib, shape, periodic, messages):
    """ni < 0 in the reference: only points on a subdomain boundary are summed."""
    O, F = oracle, faces_lib
    s = O.Shape(*shape, periodic=periodic)
    u_init, out, chk = run_gpu(F, s, periodic=periodic, messages=messages, compute=False, nsteps=2)
    exp = O.groups_share(s, O.init_int(s, 5), False, 2)
    assert np.array_equal(out, exp)
    assert chk.passed


@pytest.mark.parametrize("shape", SHAPES[:6], ids=lambda s: "x".join(map(str, s)))
@pytest.mark.parametrize("messages", [False, True], ids=["direct", "messages"])
def test_gather_kernel(oracle, faces_lib, shape, messages):
    O, F = oracle, faces_lib
    s = O.Shape(*shape, periodic=True)
    _, out, _ = run_gpu(F, s, periodic=True, messages=messages, gather=True, init="ref", nsteps=2)
    assert np.array_equal(out, O.groups_share(s, O.init_ref(s), True, 2))


def test_mugs_bit_exact_single_rank(oracle, faces_lib):
    """One non-periodic rank: equal to the Mugs restatement (and so to the
    reference's own Mugs) bit for bit on the reference init."""
    O, F = oracle, faces_lib
    s = O.Shape(1, 1, 1, 3, 4, 2, 6)
    _, out, _ = run_gpu(F, s, periodic=False, messages=False, init="ref", nsteps=4)
    assert np.array_equal(out, O.mugs_share(s, O.init_ref(s), True, 4))


@pytest.mark.parametrize("chunk", [1, 2, 3, 5, 8, 16])
@pytest.mark.parametrize("kernel", ["tiles", "general", "rows", "seams"])
def test_chunking(oracle, faces_lib, chunk, kernel):
    O, F = oracle, faces_lib
    for periodic, messages in itertools.product([False, True], [False, True]):
        if kernel == "seams" and messages:
            continue
        s = O.Shape(2, 1, 1, 7, 2, 2, 5, periodic=periodic)
        f = F.Faces(*((s.lx, s.ly, s.lz, s.mx, s.my, s.mz, s.n)), periodic=periodic, messages=messages,
                    rows=kernel == "rows", general=kernel == "general", seams=kernel == "seams")
        f.set_tuning(chunk=chunk, width=1 + chunk % 3, order=[0, 1, 2, 2 + 16][chunk % 4])
        u = f.field()
        f.init_ref(u)
        f.share_n(u, 2)
        torch.cuda.synchronize()
        assert np.array_equal(u.cpu().numpy(), O.groups_share(s, O.init_ref(s), True, 2))


@pytest.mark.parametrize("kernel", ["tiles", "rows"])
def test_large_field_properties(oracle, faces_lib, kernel):
    """The benchmark's 48^3 n=8 periodic field: too large for the oracle in a
    test, so check size-independent properties on the device: the closed
    form after several shares, and direct mode == message mode bit for bit."""
    F = faces_lib
    outs = []
    for messages in (False, True):
        f = F.Faces(1, 1, 1, 48, 48, 48, 8, periodic=True, messages=messages, rows=kernel == "rows")
        u = f.field()
        f.init_int(u, 1)
        f.share_n(u, 6)
        chk = f.check(u, init="int", seed=1, nshares=6)
        assert chk.passed and chk.maxrel == 0.0
        outs.append(u)
        f.close()
    assert torch.equal(outs[0], outs[1])


@pytest.mark.parametrize("shape", [(1, 1, 1, 9, 7, 5, 8), (2, 1, 2, 5, 3, 4, 5), (1, 2, 1, 6, 4, 3, 10),
                                   (1, 1, 1, 6, 5, 4, 12), (2, 1, 1, 3, 4, 2, 11)],
                         ids=lambda s: "x".join(map(str, s)))
@pytest.mark.parametrize("periodic", [False, True], ids=["open", "periodic"])
def test_autotune_keeps_results(oracle, faces_lib, shape, periodic):
    """faces_autotune times several tile settings (and, at n >= 11 in direct
    mode, the seam kernel's forms) on the field and keeps one; every setting
    it can pick must give the oracle's result."""
    O, F = oracle, faces_lib
    s = O.Shape(*shape, periodic=periodic)
    f = F.Faces(*shape, periodic=periodic)
    u = f.field()
    f.init_int(u, 5)
    applied = f.autotune(u, trials=1)
    assert applied >= 4
    t = f.tuning()
    assert t["chunk"] >= 1 and t["unit_chunks"] >= 1 and t["blocks"] >= 1
    f.init_int(u, 5)
    f.share_n(u, 3)
    torch.cuda.synchronize()
    assert np.array_equal(u.cpu().numpy(), O.groups_share(s, O.init_int(s, 5), True, 3))
    f.close()


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
@pytest.mark.parametrize("periodic", [False, True], ids=["open", "periodic"])
@pytest.mark.parametrize("fused", [False, True], ids=["basic", "fused"])
def test_v6_bit_exact(oracle, faces_lib, shape, periodic, fused):
    """The v-6 strategy (six face messages, sweeps z, y, x; fused: four
    launches, gpu/v-6-messages-overlap-fusable) against the oracle's v-6
    restatement bit for bit, on both inits and with compute on and off; on
    integer inputs also against the tree of the other modes."""
    O, F = oracle, faces_lib
    s = O.Shape(*shape, periodic=periodic)
    for init in ("int", "ref"):
        for compute in (True, False):
            f = F.Faces(*shape, periodic=periodic, v6=not fused, v6f=fused)
            alone = shape[0] * shape[1] * shape[2] == 1 and not periodic  # no face message to pack
            assert f.launches_per_share() == (4 if fused else 3 if alone else 6)
            u = f.field()
            f.init_int(u, 5) if init == "int" else f.init_ref(u)
            f.share_n(u, 3, compute)
            chk = f.check(u, init=init, seed=5, nshares=3, compute=compute)
            torch.cuda.synchronize()
            out = u.cpu().numpy()
            f.close()
            ref0 = O.init_int(s, 5) if init == "int" else O.init_ref(s)
            assert np.array_equal(out, O.v6_share(s, ref0.copy(), compute, 3)), (init, compute)
            if init == "int":
                assert np.array_equal(out, O.groups_share(s, ref0.copy(), compute, 3))
            assert chk.passed, (init, compute, chk.maxrel)


@pytest.mark.parametrize("shape", [(1, 1, 1, 4, 4, 4, 5), (1, 1, 1, 3, 2, 5, 8), (3, 3, 3, 2, 2, 2, 6),
                                   (2, 2, 2, 1, 1, 1, 7), (1, 1, 1, 5, 2, 3, 10), (1, 3, 1, 3, 1, 2, 9),
                                   (2, 1, 2, 2, 2, 1, 12), (1, 1, 1, 9, 3, 2, 2), (1, 1, 1, 33, 2, 3, 3),
                                   (2, 1, 1, 7, 3, 2, 4)],
                         ids=lambda s: "x".join(map(str, s)))
def test_warp_tiles_bit_exact(oracle, faces_lib, shape):
    """Tile order 3: the periodic step with one warp per tile."""
    O, F = oracle, faces_lib
    s = O.Shape(*shape, periodic=True)
    for init in ("int", "ref"):
        f = F.Faces(*shape, periodic=True)
        f.set_tuning(order=3)
        u = f.field()
        f.init_int(u, 5) if init == "int" else f.init_ref(u)
        f.share_n(u, 3)
        torch.cuda.synchronize()
        out = u.cpu().numpy()
        f.close()
        ref0 = O.init_int(s, 5) if init == "int" else O.init_ref(s)
        assert np.array_equal(out, O.groups_share(s, ref0, True, 3)), init


@pytest.mark.parametrize("shape", [(1, 1, 1, 15, 14, 13, 12), (2, 2, 1, 9, 7, 5, 11), (1, 2, 2, 11, 6, 7, 10),
                                   (3, 1, 1, 6, 9, 8, 9), (1, 1, 1, 24, 5, 6, 3), (3, 3, 3, 16, 16, 16, 6)],
                         ids=lambda s: "x".join(map(str, s)))
@pytest.mark.parametrize("periodic", [False, True], ids=["open", "periodic"])
@pytest.mark.parametrize("mode", ["tiles", "general", "rows", "messages", "v6", "seams", "seams-lean"])
def test_larger_shapes_closed_form(faces_lib, shape, periodic, mode):
    """The reference's 15x14x13 n=12 shape, the 3x3x3-rank 16^3 n=6 grid at
    full size, and other shapes with every dimension several elements long,
    every strategy: the device closed form after 3 shares, and equality with
    the default kernel bit for bit."""
    F = faces_lib
    outs = []
    for m in ("tiles", mode):
        f = F.Faces(*shape, periodic=periodic, general=m == "general", rows=m == "rows",
                    messages=m == "messages", v6=m == "v6", seams=m.startswith("seams"))
        if m == "seams-lean":
            f.set_tuning(order=1)
        u = f.field()
        f.init_int(u, 9)
        f.share_n(u, 3)
        chk = f.check(u, init="int", seed=9, nshares=3)
        assert chk.passed and chk.maxrel == 0.0, (m, chk)
        outs.append(u)
        f.close()
    assert torch.equal(outs[0], outs[1])


@pytest.mark.parametrize("shape", [(1, 1, 1, 15, 14, 13, 12), (2, 2, 1, 9, 7, 5, 11), (3, 3, 3, 16, 16, 16, 6)],
                         ids=lambda s: "x".join(map(str, s)))
@pytest.mark.parametrize("periodic", [False, True], ids=["open", "periodic"])
@pytest.mark.parametrize("mode", ["messages", "v6", "gather"])
def test_larger_shapes_without_compute(faces_lib, shape, periodic, mode):
    """compute = 0 (the reference's ni < 0) on the larger shapes: the
    boundary-only sums of every strategy against the device closed form, and
    bit-equal to the default path."""
    F = faces_lib
    outs = []
    for m in ("tiles", mode):
        f = F.Faces(*shape, periodic=periodic, messages=m == "messages", v6=m == "v6", gather=m == "gather")
        u = f.field()
        f.init_int(u, 4)
        f.share_n(u, 2, False)
        chk = f.check(u, init="int", seed=4, nshares=2, compute=False)
        assert chk.passed and chk.maxrel == 0.0, (m, chk)
        outs.append(u)
        f.close()
    assert torch.equal(outs[0], outs[1])


@pytest.mark.parametrize("args,opts", [("1 1 1 6 5 4 8 1 2 3", ["--periodic", "--init=int", "--autotune"]),
                                       ("2 1 1 5 4 3 12 1 1 2", ["--autotune"]),
                                       ("1 1 1 4 4 4 5 1 2 -5", ["--periodic", "--autotune"])])
def test_executable_autotune(faces_lib, args, opts):
    """The drop-in executable with --autotune still prints the reference's
    pass line for every rank."""
    import subprocess
    exe = faces_lib.exe_path
    r = subprocess.run([exe] + opts, input=args + "\n", capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    nranks = int(args.split()[0]) * int(args.split()[1]) * int(args.split()[2])
    assert f"{nranks} tasks passed correctness check" in r.stdout, r.stdout


@pytest.mark.parametrize("messages", [False, True], ids=["direct", "messages"])
def test_run_host_many(oracle, faces_lib, messages):
    """faces_run_host_many (uploads and downloads overlapping the shares of
    neighbouring jobs) gives every job the result of faces_run_host alone,
    and the oracle's; in place, one job and no job work; an input that is an
    earlier job's output is refused."""
    O, F = oracle, faces_lib
    shape = (2, 1, 1, 5, 4, 3, 6)
    s = O.Shape(*shape, periodic=True)
    f = F.Faces(*shape, periodic=True, messages=messages)
    u = f.field()
    ins = []
    for seed in (1, 2, 3, 4, 5):
        f.init_int(u, seed)
        torch.cuda.synchronize()
        ins.append(u.cpu().numpy().copy())
    outs = [np.empty_like(a) for a in ins]
    f.run_host_many(ins, outs, 3)
    for seed, a, b in zip((1, 2, 3, 4, 5), ins, outs):
        alone = np.empty_like(a)
        f.run_host(a, alone, 3)
        assert np.array_equal(b, alone), seed
    assert np.array_equal(outs[2], O.groups_share(s, O.init_int(s, 3), True, 3))
    inplace = [a.copy() for a in ins[:3]]
    f.run_host_many(inplace, inplace, 3)
    for a, b in zip(inplace, outs[:3]):
        assert np.array_equal(a, b)
    one = [np.empty_like(ins[0])]
    f.run_host_many(ins[:1], one, 3)
    assert np.array_equal(one[0], outs[0])
    f.run_host_many([], [], 3)
    with pytest.raises(F.FacesError):
        f.run_host_many([ins[0], outs[0]], [outs[0], outs[1]], 3)
    f.close()


@pytest.mark.parametrize("shape", [(3, 3, 3, 4, 3, 2, 6), (2, 1, 2, 5, 3, 4, 5), (3, 3, 3, 16, 16, 16, 6),
                                   (2, 2, 1, 9, 7, 5, 11), (1, 1, 1, 6, 5, 4, 8)],
                         ids=lambda s: "x".join(map(str, s)))
@pytest.mark.parametrize("periodic", [False, True], ids=["open", "periodic"])
def test_fused_pack_equals_separate(oracle, faces_lib, shape, periodic):
    """v-26 message mode with the pack in the tile kernel's prologue
    (FACES_PACK_FUSED: one cooperative launch per share) and as its own
    launch (the default): the same bits, the oracle's, and no wait of the
    fused form ran out."""
    O, F = oracle, faces_lib
    outs = []
    for sep in (False, True):
        f = F.Faces(*shape, periodic=periodic, messages=True, pack_fused=not sep)
        # one non-periodic rank has no message: no pack launch either way
        alone = shape[0] * shape[1] * shape[2] == 1 and not periodic
        assert f.launches_per_share() == (2 if sep and not alone else 1)
        u = f.field()
        f.init_int(u, 3)
        f.share_n(u, 4)
        chk = f.check(u, init="int", seed=3, nshares=4)
        assert chk.passed and chk.maxrel == 0.0, (sep, chk)
        assert f.status() == 0
        outs.append(u)
        f.close()
    assert torch.equal(outs[0], outs[1])
    s = O.Shape(*shape, periodic=periodic)
    if s.total_doubles < 20_000_000:
        assert np.array_equal(outs[0].cpu().numpy(), O.groups_share(s, O.init_int(s, 3), True, 4))


def test_fused_pack_wait_runs_out_and_reports(faces_lib):
    """The fused step's wait is bounded: made to wait for an arrival that
    never comes (test hook), every waiting block gives up after a short
    bound, sets status bit 0 and returns; the status reads it once, and the
    same context then shares correctly again."""
    F = faces_lib
    f = F.Faces(3, 3, 3, 4, 3, 2, 6, periodic=True, messages=True, pack_fused=True)
    u = f.field()
    f.init_int(u, 3)
    f.share_n(u, 1)
    torch.cuda.synchronize()
    assert f.status() == 0
    f.test_pack_wait(1, 1 << 12)
    f.share_n(u, 1)
    torch.cuda.synchronize()
    assert f.status() == 1
    assert f.status() == 0  # read and cleared
    f.test_pack_wait(0)
    f.init_int(u, 3)
    f.share_n(u, 2)
    chk = f.check(u, init="int", seed=3, nshares=2)
    assert chk.passed and chk.maxrel == 0.0
    assert f.status() == 0
    f.close()

"""The CPU oracle (oracle/faces_oracle.c) pinned to the reference.

* golden vectors made by the reference's own gpu/Mugs.cc (tests/golden/)
* the reference's Mugs itself (oracle/_ref), where its sources are present
* three independent formulations agreeing with each other
* a pure-Python restatement on tiny shapes
"""
import hashlib
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def golden_cases():
    with open(os.path.join(GOLDEN, "golden.json")) as fh:
        return json.load(fh)["cases"]


def initial(O, s, init, seed):
    return O.init_ref(s) if init == "ref" else O.init_int(s, seed)


@pytest.mark.parametrize("case", golden_cases(), ids=lambda c: c["name"])
def test_golden_vectors(oracle, case):
    """Mugs restatement == the reference's Mugs output, bit for bit."""
    O = oracle
    s = O.Shape(*case["shape"], periodic=False)
    exp = np.load(os.path.join(GOLDEN, case["name"] + ".npz"))["out"]
    assert hashlib.sha256(exp.tobytes()).hexdigest() == case["sha256"]
    u0 = initial(O, s, case["init"], case["seed"])
    got = O.mugs_share(s, u0.copy(), case["compute"], case["shares"])
    assert np.array_equal(got, exp)
    # the tree-order formulations: exact on one rank or integer inputs, and
    # within the reference's 1e-15 check otherwise
    g = O.groups_share(s, u0.copy(), case["compute"], case["shares"])
    if s.nranks == 1 or case["init"] == "int":
        assert np.array_equal(g, exp)
    mv, npass, _ = O.compare(s, g, exp)
    assert mv < 1e-15 and npass == s.nranks


def test_reference_init_values(oracle):
    """gpu/main.cc:18: u = jz*1e4 + jy*100 + jx + iz*0.01 + iy*1e-4 + ix*1e-6."""
    O = oracle
    s = O.Shape(1, 1, 1, 3, 3, 3, 4)
    v = O.view6(s, O.init_ref(s)) if hasattr(O, "view6") else s.view6(O.init_ref(s))
    assert v[1, 1, 1, 3, 2, 1] == 10101 + 3 * 0.01 + 2 * 0.0001 + 1 * 0.000001
    assert v[2, 0, 1, 0, 0, 0] == 20001.0
    # padding stays zero (DArray zero-fills, gpu/DArray.h:77-82)
    u = O.init_ref(s)
    plane = s.n ** 3 * s.mx * s.my
    assert np.all(u.reshape(s.mz, s.jz_stride)[:, plane:] == 0)


def test_integer_init(oracle):
    O = oracle
    s = O.Shape(2, 1, 1, 3, 2, 2, 5)
    u = O.init_int(s, 42)
    plane = s.n ** 3 * s.mx * s.my
    body = u.reshape(s.nranks * s.mz, s.jz_stride)[:, :plane]
    assert np.all(body == np.floor(body)) and body.min() >= 0 and body.max() < 2 ** 20
    assert abs(body.mean() / 2 ** 19 - 1) < 0.05
    assert np.all(u.reshape(s.nranks * s.mz, s.jz_stride)[:, plane:] == 0)
    assert O.lib().orc_int_value(42, 7) == u[7]


REF_SHAPES = [(1, 1, 1, 3, 2, 4, 5), (2, 1, 1, 2, 3, 2, 4), (2, 2, 2, 2, 2, 2, 3), (3, 1, 2, 2, 1, 3, 6),
              (1, 1, 1, 1, 1, 1, 3), (1, 1, 1, 2, 2, 2, 2), (2, 3, 1, 1, 2, 1, 4), (1, 2, 1, 2, 2, 3, 7)]


@pytest.mark.parametrize("shape", REF_SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_against_reference_mugs(oracle, shape):
    """The reference's own Mugs (built here from its sources) on random inputs."""
    O = oracle
    if not O.ref_available():
        pytest.skip("reference sources not present: oracle/_ref not built (golden vectors cover this)")
    s = O.Shape(*shape)
    rng = np.random.default_rng(sum(shape))
    for compute in (True, False):
        u0 = O.init_int(s, 5)
        m = u0 != 0
        u0[m] = rng.standard_normal(m.sum())
        exp = O.ref_mugs_share(s, u0.copy(), compute, 3)
        assert np.array_equal(O.mugs_share(s, u0.copy(), compute, 3), exp)
        if s.nranks == 1:
            assert np.array_equal(O.groups_share(s, u0.copy(), compute, 3), exp)


@pytest.mark.parametrize("periodic", [False, True], ids=["open", "periodic"])
@pytest.mark.parametrize("shape", REF_SHAPES + [(3, 3, 3, 2, 2, 2, 3), (1, 2, 1, 1, 1, 1, 4)],
                         ids=lambda s: "x".join(map(str, s)))
def test_formulations_agree(oracle, shape, periodic):
    """global groups == v-26 pack/inner/unpack on any input; all three equal
    on integer inputs (K3: every partial sum is exact)."""
    O = oracle
    s = O.Shape(*shape, periodic=periodic)
    rng = np.random.default_rng(3)
    for compute in (True, False):
        u0 = O.init_int(s, 13)
        g = O.groups_share(s, u0.copy(), compute, 4)
        assert np.array_equal(g, O.v26_share(s, u0.copy(), compute, 4))
        assert np.array_equal(g, O.mugs_share(s, u0.copy(), compute, 4))
        m = u0 != 0
        u1 = u0.copy()
        u1[m] = rng.random(m.sum()) * 100
        assert np.array_equal(O.groups_share(s, u1.copy(), compute, 2), O.v26_share(s, u1.copy(), compute, 2))
        mv, npass, _ = O.compare(s, O.groups_share(s, u1.copy(), compute, 2), O.mugs_share(s, u1.copy(), compute, 2))
        assert mv < 1e-15


def python_share(s, u, compute=True, order="xyz"):
    """Pure-Python statement of one share on the global mesh (tiny shapes):
    every global point's copies get the sum x-pairs -> y-pairs -> z-pairs
    (order "zyx": z-pairs -> y-pairs -> x-pairs, the v-6 sweeps)."""
    n = s.n
    L, m = (s.lx, s.ly, s.lz), (s.mx, s.my, s.mz)
    M = [L[a] * m[a] for a in range(3)]
    v = u.copy()

    def copies(g, a):
        E, i = divmod(g, n - 1)
        if i:
            return [(E, i)]
        if s.periodic:
            return [((E - 1) % M[a], n - 1), (E % M[a], 0)]
        if E == 0:
            return [(0, 0)]
        if E == M[a]:
            return [(M[a] - 1, n - 1)]
        return [(E - 1, n - 1), (E, 0)]

    def addr(E, i):
        k = [E[a] // m[a] for a in range(3)]
        j = [E[a] % m[a] for a in range(3)]
        r = (k[2] * s.ly + k[1]) * s.lx + k[0]
        return (r * s.rank_doubles + i[0] + n * i[1] + n * n * i[2] + n ** 3 * j[0]
                + n ** 3 * s.mx * j[1] + s.jz_stride * j[2])

    G = [M[a] * (n - 1) + (0 if s.periodic else 1) for a in range(3)]
    for gz in range(G[2]):
        for gy in range(G[1]):
            for gx in range(G[0]):
                cx, cy, cz = copies(gx, 0), copies(gy, 1), copies(gz, 2)
                if len(cx) * len(cy) * len(cz) == 1:
                    continue
                span = [m[a] * (n - 1) for a in range(3)]
                if not compute and all(g % sp for g, sp in zip((gx, gy, gz), span)):
                    continue
                def pair(v):
                    return v[0] + v[1] if len(v) == 2 else v[0]

                def val(ex, ey, ez):
                    return u[addr((ex[0], ey[0], ez[0]), (ex[1], ey[1], ez[1]))]

                if order == "xyz":
                    tot = pair([pair([pair([val(ex, ey, ez) for ex in cx]) for ey in cy]) for ez in cz])
                else:
                    tot = pair([pair([pair([val(ex, ey, ez) for ez in cz]) for ey in cy]) for ex in cx])
                for ez in cz:
                    for ey in cy:
                        for ex in cx:
                            v[addr((ex[0], ey[0], ez[0]), (ex[1], ey[1], ez[1]))] = tot
    return v


@pytest.mark.parametrize("shape,periodic", [((1, 1, 1, 2, 2, 2, 3), True), ((2, 1, 1, 2, 1, 2, 3), False),
                                            ((1, 2, 2, 1, 2, 1, 4), True), ((2, 2, 2, 1, 1, 1, 2), True)])
def test_pure_python_restatement(oracle, shape, periodic):
    O = oracle
    s = O.Shape(*shape, periodic=periodic)
    rng = np.random.default_rng(0)
    u0 = O.init_int(s, 2)
    m = u0 != 0
    u0[m] = rng.standard_normal(m.sum())
    for compute in (True, False):
        assert np.array_equal(python_share(s, u0, compute), O.groups_share(s, u0.copy(), compute, 1))


@pytest.mark.parametrize("shape,periodic", [((1, 1, 1, 2, 2, 2, 3), True), ((2, 1, 1, 2, 1, 2, 3), False),
                                            ((1, 2, 2, 1, 2, 1, 4), True), ((2, 2, 2, 1, 1, 1, 2), True),
                                            ((2, 1, 2, 3, 1, 1, 2), False)])
def test_v6_restatement(oracle, shape, periodic):
    """The v-6 sweeps (z, then y, then x) give every point the tree sum in the
    order z pairs, y pairs, x pairs; on integer inputs that equals every other
    formulation."""
    O = oracle
    s = O.Shape(*shape, periodic=periodic)
    rng = np.random.default_rng(1)
    u0 = O.init_int(s, 2)
    for compute in (True, False):
        assert np.array_equal(O.v6_share(s, u0.copy(), compute, 3), O.groups_share(s, u0.copy(), compute, 3))
    m = u0 != 0
    u1 = u0.copy()
    u1[m] = rng.standard_normal(m.sum())
    for compute in (True, False):
        assert np.array_equal(python_share(s, u1, compute, order="zyx"), O.v6_share(s, u1.copy(), compute, 1))


@pytest.mark.parametrize("periodic", [False, True], ids=["open", "periodic"])
def test_v6_reference_init_within_check(oracle, periodic):
    """On the reference's non-integer init the v-6 order differs from Mugs in
    the last bits only: within the reference's own 1e-15 check."""
    O = oracle
    s = O.Shape(2, 2, 1, 3, 2, 4, 5, periodic=periodic)
    a = O.v6_share(s, O.init_ref(s), True, 3)
    b = O.mugs_share(s, O.init_ref(s), True, 3)
    mv, npass, _ = O.compare(s, a, b)
    assert mv < 1e-15 and npass == s.nranks


def test_closed_form_of_repeated_shares(oracle):
    """After s shares every copy of a point with k seam axes holds the first
    share's value times 2^(k*(s-1)) -- the property the device check uses."""
    O = oracle
    s = O.Shape(2, 1, 1, 2, 2, 2, 4, periodic=True)
    u0 = O.init_ref(s)
    one = O.groups_share(s, u0.copy(), True, 1)
    five = O.groups_share(s, u0.copy(), True, 5)
    nz = one != 0
    ratio = five[nz] / one[nz]
    assert set(np.unique(ratio)) <= {1.0, 2.0 ** 4, 4.0 ** 4, 8.0 ** 4}
    assert set(np.unique(ratio)) == {1.0, 2.0 ** 4, 4.0 ** 4, 8.0 ** 4}


def test_sum_is_conserved_per_global_point(oracle):
    """Integer inputs: the sum over all copies equals sum over points of
    copies(point) * value -- a checksum of checksums."""
    O = oracle
    s = O.Shape(1, 1, 1, 3, 3, 3, 4, periodic=True)
    u0 = O.init_int(s, 17)
    u1 = O.groups_share(s, u0.copy(), True, 1)
    v0, v1 = s.view6(u0), s.view6(u1)
    # multiplicity of each copy: 2 per seam axis
    n = s.n
    mult = np.ones((n, n, n))
    for a in range(3):
        sl = [slice(None)] * 3
        for i in (0, n - 1):
            sl[a] = i
            mult[tuple(sl)] *= 2
    mult = mult[None, None, None]  # (jz,jy,jx) broadcast; view is (jz,jy,jx,iz,iy,ix)
    assert np.sum(v1) == np.sum(v0 * mult)

"""The reference's Riemann known-answer states, clamped states and boundary
fluxes through the device flux code, and the kernels' hand-written
arithmetic against CUDA's own operators.

The face kernels of every scheme evaluate `interior_flux_weighted` and
`flux_boundary` (csrc/euler.cuh); `mcfd_probe_flux` runs the same template
instances (solver x FP64 / mixed form) on given states.  Checked here:

* every KAT of test/riemann/euler/{exact,hllc,ausm}.cpp (Sod, the blast
  waves, shock collision, the 123 problem, near vacuum, left / right
  vacuum; transcribed in tests/golden/riemann_kat.json) against the
  reference's expected Godunov state with the reference test's tolerance,
  for the solver the KAT names, in both forms and at random face
  orientations;
* the same states through all five solvers against the oracle
  (oracle/orc_gas.c, the rotated-solver restatement), with states that
  SetZeroIfNegative clamps (riemann/euler/types.hpp:194-202) on either side;
* every boundary kind (rotated/euler.hpp:144-318) against the oracle;
* rcp_newton / rcp_signed (Newton reciprocals from an FP32 seed) within one
  ulp of CUDA's correctly rounded 1.0 / x over the whole exponent range and
  at the seed guards; rcp_newton1 (one Newton step, the mixed form's node
  traces) and sqrt_seeded within their stated relative bounds of 1.0 / x and
  sqrt; f64_to_f32 / f32_to_f64 bit-equal to __double2float_rn and
  (double)f except the stated flush of magnitudes below 2^-126 to a signed
  zero (NaN stays NaN, infinities stay infinite).
"""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

import oracle.orc as orc
from pvcriemannsolvers_gb300 import capi

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
KAT = json.loads((GOLDEN / "riemann_kat.json").read_text())
SOLVERS = {"exact": capi.EXACT, "hllc": capi.HLLC, "ausm": capi.AUSM, "roe": capi.ROE,
           "rusanov": capi.RUSANOV}
FORMS = {"fp64": capi.FP64, "mixed": capi.MIXED}
ORC_KIND = {capi.EXACT: orc.EXACT, capi.HLLC: orc.HLLC, capi.AUSM: orc.AUSM, capi.ROE: orc.ROE,
            capi.RUSANOV: orc.RUSANOV}
G = 1.4


def to3d(state, dim):
    s = list(state)
    if dim == 1:
        return [s[0], s[1], 0.0, 0.0, s[2]]
    if dim == 2:
        return [s[0], s[1], s[2], 0.0, s[3]]
    return s


def flux_of(prim):
    """Normal-frame physical flux of a primitive state (types.hpp:312-321)."""
    rho, u, v, w, p = prim
    e = p / (G - 1) + 0.5 * rho * (u * u + v * v + w * w)
    return np.array([rho * u, rho * u * u + p, rho * v * u, rho * w * u, (e + p) * u])


def components(dim):
    return {1: [0, 1, 4], 2: [0, 1, 2, 4], 3: [0, 1, 2, 3, 4]}[dim]


def frame_of(n, rng=None):
    """Orthonormal rows (n, t, b), as a face's Riemann frame."""
    n = np.asarray(n, float) / np.linalg.norm(n)
    a = np.array([0.3, 0.7, 0.2]) if rng is None else rng.normal(size=3)
    t = np.cross(n, a)
    t /= np.linalg.norm(t)
    return np.stack([n, t, np.cross(n, t)])


def prim_to_global_cons(prim_normal, frame):
    """A state given in the face frame (u_n, u_t, u_b) -> global conservative."""
    rho, un, ut, ub, p = prim_normal
    vel = frame.T @ np.array([un, ut, ub])
    return orc.prim_to_cons([rho, *vel, p])


def probe_flux(riemann, form, left, right, normals, bc_kind=capi.BC_NONE):
    """Device flux for the rows of left / right / normals ([n][5], [n][5], [n][3])."""
    import torch
    lib = capi.load()
    l = torch.from_numpy(np.ascontiguousarray(left, dtype=np.float64)).cuda()
    r = torch.from_numpy(np.ascontiguousarray(right, dtype=np.float64)).cuda()
    nv = torch.from_numpy(np.ascontiguousarray(normals, dtype=np.float64)).cuda()
    n = l.shape[0]
    f = torch.full((n, 5), float("nan"), dtype=torch.float64, device="cuda")
    status = C.c_uint32(0)
    code = lib.mcfd_probe_flux(0, riemann, form, bc_kind, n, C.c_void_p(l.data_ptr()),
                               C.c_void_p(r.data_ptr()), C.c_void_p(nv.data_ptr()),
                               C.c_void_p(f.data_ptr()), C.byref(status))
    assert code in (capi.OK, capi.ERR_NOT_CONVERGED), code
    return f.cpu().numpy(), status.value


def assert_matches_oracle(got, want, tol, what):
    """Row-wise: the same non-finite components, and finite ones within
    tol x (1 + |want row|_inf)."""
    for i in range(want.shape[0]):
        g, w = got[i], want[i]
        assert np.array_equal(np.isfinite(g), np.isfinite(w)), (what, i, g, w)
        fin = np.isfinite(w)
        scale = 1.0 + (np.max(np.abs(w[fin])) if fin.any() else 0.0)
        err = np.max(np.abs(g[fin] - w[fin])) if fin.any() else 0.0
        assert err <= tol * scale, (what, i, err / scale, g, w)


def tolerance(riemann, form):
    if riemann == capi.EXACT:
        return 1e-10  # the root finder stops at |f| < 1e-8 (exact.hpp:140-152)
    if form == capi.MIXED and riemann in (capi.HLLC, capi.ROE, capi.RUSANOV):
        return 1e-11  # seeded square roots, relative error below 2e-13
    return 1e-12


ALL_CASES = [(c["solver"], c["dim"], c["left"], c["right"], c) for c in KAT["cases"]]


@pytest.mark.parametrize("form", list(FORMS))
@pytest.mark.parametrize("case", ALL_CASES,
                         ids=lambda c: f"{c[0]}{c[1]}d:{c[4]['src'].split('/')[-1]}:{c[4]['line']}")
def test_kat_through_device_flux(gpu, case, form):
    """The Godunov state the reference's KAT expects, at the identity frame
    and at 16 random face orientations (the flux rotated back to the face
    frame), with the reference test's tolerance."""
    solver, dim, left, right, c = case
    rng = np.random.default_rng(c["line"])
    frames = [np.eye(3)] + [frame_of(rng.normal(size=3), rng) for _ in range(16)]
    lw, rw = to3d(left, dim), to3d(right, dim)
    L = np.array([prim_to_global_cons(lw, f) for f in frames])
    R = np.array([prim_to_global_cons(rw, f) for f in frames])
    N = np.array([f[0] for f in frames])
    got, _ = probe_flux(SOLVERS[solver], FORMS[form], L, R, N)
    want = flux_of(to3d(c["expect"], dim))
    scale = 1.0 + np.max(np.abs(want))
    for i, f in enumerate(frames):
        g = got[i].copy()
        g[1:4] = f @ g[1:4]  # momentum flux back into the face frame
        for j, comp in enumerate(components(dim)):
            eps = c["eps"][j]
            x, y = want[comp], g[comp]
            if x == 0:
                # an exact zero of the KAT; rotating to and from a random
                # frame leaves rounding of the flux's size
                assert abs(y) <= 1e-13 * scale, (i, comp, x, y)
            elif c["cmp"] == "near":
                assert abs(y / x - 1) <= eps, (i, comp, x, y)
            else:
                assert abs(x - y) / max(abs(x), abs(y)) <= eps, (i, comp, x, y)


@pytest.mark.parametrize("form", list(FORMS))
@pytest.mark.parametrize("case", KAT["vacuum"], ids=lambda c: f"vacuum:{c['line']}")
def test_exact_vacuum_kat_through_device_flux(gpu, case, form):
    """Left / right vacuum of test/riemann/euler/exact.cpp:85-125, 290-330:
    the Exact solver's vacuum branches on the device, with the reference's
    absolute tolerances."""
    dim = case["dim"]
    lw, rw = to3d(case["left"], dim), to3d(case["right"], dim)
    L = orc.prim_to_cons(lw)[None]
    R = orc.prim_to_cons(rw)[None]
    got, status = probe_flux(capi.EXACT, FORMS[form], L, R, np.array([[1.0, 0.0, 0.0]]))
    assert status == 0
    if case["expect"] == "left":
        want = flux_of(lw)
    elif case["expect"] == "right":
        want = flux_of(rw)
    else:
        want = flux_of(to3d(case["expect"], dim))
    # The reference's absolute tolerance on the Godunov state, or a relative
    # one for the flux assembled from it.  The device takes conservative
    # inputs and recovers p = (gamma - 1)(E - |m|^2 / 2 rho), whose condition
    # number is E / (rho e): 817 for the state of exact.cpp:320 (tangential
    # speed 54 against a sound speed of 1), so rounding of the inputs reaches
    # the result amplified by that factor.
    kappa = max(input_condition(w) for w in (lw, rw))
    rel = max(1e-14, 16 * np.finfo(float).eps * kappa)
    for comp in components(dim):
        assert abs(got[0, comp] - want[comp]) <= max(case["atol"], rel * abs(want[comp])), \
            (comp, got[0], want)


def input_condition(prim):
    """E / (rho e) of a primitive state: the amplification of relative
    rounding in the conservative variables into the recovered pressure."""
    rho, u, v, w, p = prim
    if rho <= 0 or p <= 0:
        return 1.0
    internal = p / (G - 1)
    return (internal + 0.5 * rho * (u * u + v * v + w * w)) / internal


def kat_state_pairs():
    """Every KAT and vacuum state pair, as (left prim, right prim) in 3D."""
    pairs = [(to3d(c["left"], c["dim"]), to3d(c["right"], c["dim"])) for c in KAT["cases"]]
    pairs += [(to3d(c["left"], c["dim"]), to3d(c["right"], c["dim"])) for c in KAT["vacuum"]]
    return pairs


def clamped_cons_states():
    """Conservative states that ConservativeToPrimitive + SetZeroIfNegative
    turns into the zero state: negative density, negative energy, negative
    pressure (kinetic energy above E), the vacuum (0, 0, 0, 0, 0), and zero
    density with non-zero momentum or energy, which the conversion leaves
    unconverted (velocity = momentum, p = E, types.hpp:288-301)."""
    return [np.array(s, float) for s in (
        [-0.1, 0.0, 0.0, 0.0, 1.0],
        [1.0, 0.2, 0.0, 0.0, -0.5],
        [1.0, 3.0, 1.0, 0.0, 2.0],
        [0.5, -2.0, 0.5, 1.0, 0.1],
        [0.0, 0.0, 0.0, 0.0, 0.0],
        [0.0, 0.0, 0.0, 0.0, 0.5],
        [0.0, 0.3, -0.1, 0.0, 0.5],
        [1e-300, 0.0, 0.0, 0.0, 1e-300],
    )]


def oracle_pairs():
    rng = np.random.default_rng(11)
    L, R, N, F = [], [], [], []
    for lw, rw in kat_state_pairs():
        for k in range(4):
            f = np.eye(3) if k == 0 else frame_of(rng.normal(size=3), rng)
            L.append(prim_to_global_cons(lw, f))
            R.append(prim_to_global_cons(rw, f))
            N.append(f[0])
            F.append(f)
    good = orc.prim_to_cons([1.0, 0.3, -0.2, 0.1, 1.0])
    for bad in clamped_cons_states():
        for l, r in ((bad, good), (good, bad), (bad, bad)):
            f = frame_of(rng.normal(size=3), rng)
            L.append(l)
            R.append(r)
            N.append(f[0])
            F.append(f)
    return np.array(L), np.array(R), np.array(N), F


@pytest.mark.parametrize("form", list(FORMS))
@pytest.mark.parametrize("solver", list(SOLVERS))
def test_all_solvers_on_kat_and_clamped_states_match_oracle(gpu, solver, form):
    """Every solver (Roe and Rusanov included, which have no C++ KAT) on the
    KAT states at rotated frames and on clamped states against the oracle;
    non-finite results must appear in the same components."""
    L, R, N, F = oracle_pairs()
    riemann = SOLVERS[solver]
    got, _ = probe_flux(riemann, FORMS[form], L, R, N)
    want = np.array([orc.flux_rotated(ORC_KIND[riemann], F[i], L[i], R[i]) for i in range(len(F))])
    assert_matches_oracle(got, want, tolerance(riemann, FORMS[form]), solver)


BC_GIVEN = {
    capi.BC_INVISCID_WALL: None,
    capi.BC_SUPERSONIC_INLET: orc.prim_to_cons([1.2, 2.5, 0.3, -0.2, 0.8]),
    capi.BC_SUPERSONIC_OUTLET: None,
    capi.BC_SUBSONIC_INLET: np.array([1.3, 0.8, 0.6, 0.0, 1.1 / 287.05]),  # p0, cosines, T0
    capi.BC_SUBSONIC_OUTLET: np.array([0.0, 0.0, 0.0, 0.0, 0.7]),          # p in slot 4
    capi.BC_SMART: orc.prim_to_cons([0.125, 0.0, 0.1, 0.0, 0.1]),
}


@pytest.mark.parametrize("form", list(FORMS))
@pytest.mark.parametrize("solver", list(SOLVERS))
@pytest.mark.parametrize("kind", list(BC_GIVEN), ids=lambda k: f"bc{k}")
def test_boundary_fluxes_match_oracle(gpu, kind, solver, form):
    """The boundary fluxes on interior states drawn from the KATs (including
    strong shocks and near-vacuum states) at random face orientations."""
    rng = np.random.default_rng(100 + kind)
    ins, frames = [], []
    for lw, rw in kat_state_pairs():
        for w in (lw, rw):
            if w[0] <= 0:
                continue
            f = frame_of(rng.normal(size=3), rng)
            ins.append(prim_to_global_cons(w, f))
            frames.append(f)
    ins = np.array(ins)
    given = BC_GIVEN[kind]
    G_ = np.zeros_like(ins) if given is None else np.tile(given, (len(ins), 1))
    N = np.array([f[0] for f in frames])
    riemann = SOLVERS[solver]
    got, _ = probe_flux(riemann, FORMS[form], ins, G_, N, bc_kind=kind)
    want = np.array([orc.flux_boundary(ORC_KIND[riemann], kind, frames[i], ins[i], G_[i])
                     for i in range(len(frames))])
    assert_matches_oracle(got, want, tolerance(riemann, FORMS[form]), (kind, solver))


# ---------------------------------------------------------------- numerics

def probe_numerics(op, x, out_dtype):
    import torch
    lib = capi.load()
    t_in = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    t_out = torch.empty(t_in.shape[0], dtype=out_dtype, device="cuda")
    code = lib.mcfd_probe_numerics(0, op, t_in.shape[0], C.c_void_p(t_in.data_ptr()),
                                   C.c_void_p(t_out.data_ptr()))
    assert code == capi.OK
    return t_out.cpu().numpy()


def f64_from_fields(sign, ex, mant):
    bits = (np.uint64(sign) << np.uint64(63)) | (ex.astype(np.uint64) << np.uint64(52)) | mant.astype(np.uint64)
    return bits.view(np.float64)


def f64_sweep(rng, positive_only=False):
    """Every binary64 exponent field (subnormals, 0 and inf/NaN included)
    with the extreme mantissas and random ones, both signs."""
    ex = np.repeat(np.arange(0, 2048, dtype=np.uint64), 8)
    mant = np.tile(np.array([0, 1, (1 << 52) - 1, 1 << 51, (1 << 29) - 1, 1 << 29,
                             (1 << 28), (1 << 28) + 1], dtype=np.uint64), 2048)
    rnd_ex = rng.integers(0, 2048, 40000).astype(np.uint64)
    rnd_m = rng.integers(0, 1 << 52, 40000, dtype=np.uint64)
    ex = np.concatenate([ex, rnd_ex])
    mant = np.concatenate([mant, rnd_m])
    xs = [f64_from_fields(0, ex, mant)]
    if not positive_only:
        xs.append(f64_from_fields(1, ex, mant))
    return np.concatenate(xs)


def ulp(x):
    return np.spacing(np.abs(x))


def guard_values():
    """Inputs around the seed guards: FP32-rebased exponents e = 0..3 and
    251..254, i.e. binary64 exponent fields 896..899 and 1147..1150."""
    out = []
    for ex in list(range(894, 901)) + list(range(1145, 1152)):
        for m in (0, 1, (1 << 52) - 1, 1 << 51, 0x123456789ABCD):
            out.append(f64_from_fields(0, np.array([ex], dtype=np.uint64), np.array([m], dtype=np.uint64))[0])
    return np.array(out)


def test_rcp_newton_within_one_ulp_of_cuda_division(gpu):
    import torch
    rng = np.random.default_rng(5)
    x = np.concatenate([f64_sweep(rng, positive_only=True), guard_values()])
    got = probe_numerics(capi.PROBE_RCP, x, torch.float64)
    cuda = probe_numerics(capi.PROBE_CUDA_RCP, x, torch.float64)
    with np.errstate(divide="ignore", over="ignore", invalid="ignore"):
        ref = 1.0 / x
    # CUDA's FP64 division is correctly rounded, as IEEE division on the host
    assert np.array_equal(cuda, ref, equal_nan=True)
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(got), nan)
    inf = np.isinf(ref)
    assert np.array_equal(got[inf], ref[inf])
    fin = ~nan & ~inf
    err = np.abs(got[fin] - ref[fin])
    bad = err > ulp(ref[fin])
    assert not bad.any(), (x[fin][bad][:5], got[fin][bad][:5], ref[fin][bad][:5])


def test_rcp_signed_within_one_ulp_of_cuda_division(gpu):
    import torch
    rng = np.random.default_rng(6)
    g = guard_values()
    x = np.concatenate([f64_sweep(rng), g, -g, [0.0, -0.0, np.inf, -np.inf]])
    got = probe_numerics(capi.PROBE_RCP_SIGNED, x, torch.float64)
    with np.errstate(divide="ignore", over="ignore", invalid="ignore"):
        ref = 1.0 / x
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(got), nan)
    inf = np.isinf(ref)
    assert np.array_equal(got[inf], ref[inf])
    fin = ~nan & ~inf
    assert np.array_equal(np.signbit(got[fin]), np.signbit(ref[fin]))
    err = np.abs(got[fin] - ref[fin])
    bad = err > ulp(ref[fin])
    assert not bad.any(), (x[fin][bad][:5], got[fin][bad][:5], ref[fin][bad][:5])


ROOT_RTOL = 2e-14  # two Newton steps on an FP32 seed, then up to seven roundings


def seeded_root_range(x):
    """Inputs that the Exact solver's inverse roots take: positive normal x
    with 2^-120 <= x < 2^121 (binary64 exponent fields 903..1143)."""
    ex = (x.view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF)
    return (x > 0) & (ex >= 903) & (ex <= 1143)


@pytest.mark.parametrize("op, cuda_op, what", [
    (capi.PROBE_ROOT7, capi.PROBE_CUDA_POW_ROOT7, "x^(1/7)"),
    (capi.PROBE_ROOT7_OVER_X, capi.PROBE_CUDA_POW_ROOT7, "x^(1/7) / x"),
    (capi.PROBE_POW_NEG_GAMMA, capi.PROBE_CUDA_POW_NEG_GAMMA, "x^-gamma"),
])
def test_exact_solver_roots_within_their_bound_of_cuda_pow(gpu, op, cuda_op, what):
    """The Exact solver's powers (gamma = 1.4: r^(1/7) of the expansion
    branch, its derivative's r^(1/7) / r, the isentrope's rho^-gamma) from
    FP32-seeded inverse roots: within ROOT_RTOL of CUDA's pow over the seeded
    range, and CUDA's pow itself (bit for bit) outside it: zero, subnormals,
    the extreme exponents, infinities, NaN and negative inputs."""
    import torch
    rng = np.random.default_rng(12)
    dense = 2.0 ** rng.uniform(-120, 121, 30000)
    x = np.concatenate([f64_sweep(rng), dense,
                        [0.0, -0.0, np.inf, -np.inf, np.nan, 1.0, 2.0 ** -120, 2.0 ** 121]])
    got = probe_numerics(op, x, torch.float64)
    ref = probe_numerics(cuda_op, x, torch.float64)
    if op == capi.PROBE_ROOT7_OVER_X:
        with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
            ref = ref / x
    inside = seeded_root_range(x)
    assert inside.sum() > 30000
    rel = np.abs(got[inside] - ref[inside]) / np.abs(ref[inside])
    assert rel.max() <= ROOT_RTOL, (what, rel.max(), x[inside][np.argmax(rel)])
    assert np.array_equal(got[~inside], ref[~inside], equal_nan=True), what


RCP1_RTOL = 4e-14  # one Newton step on an FP32 seed of relative error < 1.8e-7


def test_rcp_newton1_within_its_bound_of_cuda_division(gpu):
    """The mixed form's node-trace reciprocal (one Newton step): within its
    stated relative bound of CUDA's 1.0 / x over the exponent range, the
    FP64 division itself outside the seed's range."""
    import torch
    rng = np.random.default_rng(8)
    x = np.concatenate([f64_sweep(rng, positive_only=True), guard_values()])
    got = probe_numerics(capi.PROBE_RCP1, x, torch.float64)
    with np.errstate(divide="ignore", over="ignore", invalid="ignore"):
        ref = 1.0 / x
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(got), nan)
    special = nan | np.isinf(ref) | (ref == 0)
    assert np.array_equal(got[special & ~nan], ref[special & ~nan])
    fin = ~special
    rel = np.abs(got[fin] - ref[fin]) / np.abs(ref[fin])
    assert rel.max() <= RCP1_RTOL, (rel.max(), x[fin][np.argmax(rel)])
    ex = (x.view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF)
    outside = fin & ((ex <= 897) | (ex >= 1149))
    assert np.array_equal(got[outside], ref[outside])


SQRT_SEEDED_RTOL = 2e-13  # one Newton step on an FP32 seed of relative error < 3e-7


def test_sqrt_seeded_within_its_bound_of_cuda_sqrt(gpu):
    import torch
    rng = np.random.default_rng(7)
    x = np.concatenate([f64_sweep(rng, positive_only=True), guard_values(), [0.0, -0.0]])
    got = probe_numerics(capi.PROBE_SQRT_SEEDED, x, torch.float64)
    cuda = probe_numerics(capi.PROBE_CUDA_SQRT, x, torch.float64)
    ref = np.sqrt(x)
    assert np.array_equal(cuda, ref, equal_nan=True)  # correctly rounded
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(got), nan)
    special = nan | np.isinf(ref) | (ref == 0)
    assert np.array_equal(got[special & ~nan], ref[special & ~nan])
    fin = ~special
    rel = np.abs(got[fin] - ref[fin]) / ref[fin]
    assert rel.max() <= SQRT_SEEDED_RTOL, (rel.max(), x[fin][np.argmax(rel)])
    # outside the seed's range (FP32-rebased exponent <= 1 or >= 253) the
    # FP64 square root itself is used
    ex = (x.view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF)
    e32 = ex.astype(np.int64) - 896
    outside = (e32 <= 1) | (e32 >= 253)
    assert np.array_equal(got[outside], ref[outside], equal_nan=True)


def test_f64_to_f32_bit_equal_to_cuda_conversion_except_flush(gpu):
    import torch
    rng = np.random.default_rng(8)
    x = f64_sweep(rng)
    # ties and near-ties of the 29 dropped bits in the normal FP32 range
    ex = rng.integers(897, 1151, 20000).astype(np.uint64)
    hi = rng.integers(0, 1 << 23, 20000).astype(np.uint64) << np.uint64(29)
    low = np.tile(np.array([1 << 28, (1 << 28) - 1, (1 << 28) + 1, 0, (1 << 29) - 1], dtype=np.uint64), 4000)
    x = np.concatenate([x, f64_from_fields(0, ex, hi | low), f64_from_fields(1, ex, hi | low)])
    got = probe_numerics(capi.PROBE_F64_TO_F32, x, torch.float32)
    cuda = probe_numerics(capi.PROBE_CUDA_F64_TO_F32, x, torch.float32)
    with np.errstate(over="ignore"):
        ref = x.astype(np.float32)  # round to nearest even
    nan = np.isnan(x)
    assert np.array_equal(np.isnan(cuda), nan) and np.array_equal(np.isnan(got), nan)
    assert np.array_equal(cuda[~nan].view(np.uint32), ref[~nan].view(np.uint32))
    # stated difference: magnitudes below 2^-126 become a zero of x's sign
    tiny = np.abs(x) < np.float64(2.0 ** -126)
    want = ref.copy()
    want[tiny] = np.where(np.signbit(x[tiny]), np.float32(-0.0), np.float32(0.0))
    assert np.array_equal(got[~nan].view(np.uint32), want[~nan].view(np.uint32))


def test_f32_to_f64_bit_equal_to_cuda_conversion_except_flush(gpu):
    import torch
    rng = np.random.default_rng(9)
    ex = np.repeat(np.arange(0, 256, dtype=np.uint32), 6)
    mant = np.tile(np.array([0, 1, (1 << 23) - 1, 1 << 22, 0x2AAAAA, 0x155555], dtype=np.uint32), 256)
    bits = np.concatenate([ex << np.uint32(23) | mant, rng.integers(0, 1 << 32, 20000, dtype=np.uint64).astype(np.uint32)])
    bits = np.concatenate([bits, bits | np.uint32(0x80000000)])
    x = bits.view(np.float32)
    got = probe_numerics(capi.PROBE_F32_TO_F64, x, torch.float64)
    cuda = probe_numerics(capi.PROBE_CUDA_F32_TO_F64, x, torch.float64)
    ref = x.astype(np.float64)
    nan = np.isnan(x)
    assert np.array_equal(np.isnan(cuda), nan) and np.array_equal(np.isnan(got), nan)
    assert np.array_equal(cuda[~nan].view(np.uint64), ref[~nan].view(np.uint64))
    sub = (bits & np.uint32(0x7F800000)) == 0  # FP32 zeros and subnormals
    want = ref.copy()
    want[sub] = np.where(np.signbit(x[sub]), -0.0, 0.0)
    assert np.array_equal(got[~nan].view(np.uint64), want[~nan].view(np.uint64))

"""Pin the CPU oracle against outputs of the reference itself (golden fixtures).

The fixtures were produced by ``tests/golden/make_golden.py`` running the
reference's own torch code on CPU.  The finite-difference parts must match
bit for bit (same IEEE operations in the same order); spectral steps match to
the FFT library's rounding.
"""

import numpy as np
import pytest
import torch

import oracle
from conftest import load_golden, parse_bc


def t32(a):
    return torch.tensor(np.asarray(a), dtype=torch.float32).unsqueeze(0) if np.asarray(a).ndim == 3 \
        else torch.tensor(np.asarray(a), dtype=torch.float32)


def test_pad_mixed_matches_reference_test_golden():
    g = load_golden("pad_mixed")
    u = torch.tensor(g["u"])
    got = oracle.pad_bc(u, (("dirichlet", (10.0, 20.0)), "neumann", "periodic"))
    np.testing.assert_array_equal(got.numpy(), g["padded"])
    # the literal expectation of the reference's own test (tests/test_solvers.py:119-126)
    expected = np.pad(np.arange(1, 9, dtype=np.float32).reshape(2, 2, 2), 1, mode="wrap")
    expected[0, :, :] = 2.0 * 10.0 - expected[1, :, :]
    expected[-1, :, :] = 2.0 * 20.0 - expected[-2, :, :]
    expected[:, 0, :] = expected[:, 1, :]
    expected[:, -1, :] = expected[:, -2, :]
    np.testing.assert_array_equal(got.numpy()[0], expected)


@pytest.mark.parametrize("i", range(5))
def test_ch_rhs_bitexact(i):
    g = load_golden(f"ch_rhs_{i}")
    u = t32(g["u0"])
    r = oracle.ch_rhs(u, 3.0, 1.0, parse_bc(g["bc"]), tuple(g["spacing"].tolist()))
    np.testing.assert_array_equal(r.numpy(), g["rhs"])


@pytest.mark.parametrize("i", range(5))
def test_fd_forward_euler_bitexact(i):
    g = load_golden(f"fd_fe_{i}")
    u = oracle.rd_fe_run(t32(g["u0"]), int(g["n"]), float(g["dt"]), 1.0, parse_bc(g["bc"]))
    np.testing.assert_array_equal(u.numpy(), g["u"])


@pytest.mark.parametrize("i", range(4))
def test_ch_imex_matches_reference(i):
    g = load_golden(f"ch_imex_{i}")
    u = oracle.ch_imex_run(t32(g["u0"]), int(g["n"]), float(g["dt"]), float(g["eps"]), float(g["D"]))
    # same torch FFT backend on the same machine class: agreement to fp32 rounding
    assert oracle.rel_to_max(u.numpy(), g["u"]) < 1e-6


@pytest.mark.parametrize("i", range(4))
def test_ch_imex_nonperiodic_x_matches_reference(i):
    """Mirrored-x spectral step (Neumann: even extension, Dirichlet: odd) vs the reference."""
    g = load_golden(f"ch_imex_nx_{i}")
    bc = parse_bc(g["bc"])
    u = oracle.ch_imex_run(t32(g["u0"]), int(g["n"]), float(g["dt"]), float(g["eps"]), float(g["D"]), bc=bc)
    assert oracle.rel_to_max(u.numpy(), g["u"]) < 1e-6
    u64 = oracle.ch_imex_run(torch.tensor(g["u0"]).unsqueeze(0), int(g["n"]), float(g["dt"]), float(g["eps"]),
                             float(g["D"]), bc=bc)
    assert oracle.rel_to_max(g["u"], u64.numpy()) < 1e-6


@pytest.mark.parametrize("i", range(5))
def test_allen_cahn_rhs_and_rk4_match_reference(i):
    """TwoPhaseAllenCahn.rhs (19-point normal Laplacian) and three RungeKutta4 steps, bit-exact."""
    g = load_golden(f"ac_{i}")
    bc = parse_bc(g["bc"])
    kw = eval(str(g["kw"]))   # the fixture's own repr of the keyword dict
    kw.pop("bc", None)
    u0 = t32(g["u0"])
    r = oracle.ac_rhs(u0, bc=bc, **kw)
    assert np.array_equal(r.numpy(), g["rhs"])
    v = u0
    for _ in range(3):
        v = oracle.rk4_step(v, 0.1, lambda w: oracle.ac_rhs(w, bc=bc, **kw))
    assert np.array_equal(v.numpy(), g["u3"])


def rkc_case(g, dtype=torch.float32):
    """(rhs function, kwargs of the scheme) of an ``rkc_*`` fixture."""
    bc = parse_bc(g["bc"])
    kw = eval(str(g["kw"]))   # the fixture's own repr of the keyword dict
    kw.pop("bc", None)
    pname = str(g["problem"])
    if pname == "TwoPhaseAllenCahn":
        fn = lambda w: oracle.ac_rhs(w, bc=bc, **kw)  # noqa: E731
    elif pname == "ReactionDiffusion":
        fn = lambda w: oracle.rd_rhs(w, D=kw["D"], bc=bc)  # noqa: E731
    else:
        fn = lambda w: oracle.ch_rhs(w, eps=kw["eps"], D=kw["D"], bc=bc)  # noqa: E731
    return fn, eval(str(g["skw"]))


@pytest.mark.parametrize("i", range(5))
def test_rkc_matches_reference(i):
    """RKC1 / RKC2: stage coefficients and three steps over AC, RD and CH rhs."""
    g = load_golden(f"rkc_{i}")
    fn, skw = rkc_case(g)
    order = 1 if str(g["scheme"]) == "RKC1" else 2
    k32 = oracle.rkc_coeffs(order, dtype=torch.float32, **skw)
    for name, v in k32.items():   # the host's libm may differ from the fixture's by an ulp
        np.testing.assert_allclose(v.numpy(), g[name], rtol=3e-7, atol=0)
    kg = {name: torch.tensor(g[name]) for name in k32}
    v = t32(g["u0"])
    for _ in range(3):
        v = oracle.rkc_step(v, float(g["dt"]), fn, kg)
    assert np.array_equal(v.numpy(), g["u3"])
    k64 = oracle.rkc_coeffs(order, **skw)
    v = torch.tensor(g["u0"]).unsqueeze(0)
    for _ in range(3):
        v = oracle.rkc_step(v, float(g["dt"]), fn, k64)
    assert oracle.rel_to_max(v.numpy(), g["u3"]) < 1e-5


def etd1_case(g, dtype=torch.float32):
    """(symbol, rhs function, bc) of an ``etd1_*`` fixture in ``dtype``."""
    bc = parse_bc(g["bc"])
    kw = eval(str(g["kw"]))   # the fixture's own repr of the keyword dict
    kw.pop("bc", None)
    shape = tuple(int(x) for x in g["shape"])
    mirrored = oracle.x_bc_kind(bc) in ("neumann", "dirichlet")
    k2 = (oracle.rfft_k_squared_nonperiodic if mirrored else oracle.rfft_k_squared)(shape, dtype=dtype)
    pname = str(g["problem"])
    if pname == "CahnHilliard":
        sym = -2 * kw["eps"] * kw["D"] * 0.25 * k2 ** 2
        fn = lambda w: oracle.ch_rhs(w, eps=kw["eps"], D=kw["D"], bc=bc)  # noqa: E731
    elif pname == "ReactionDiffusion":
        sym = -kw["D"] * 0.25 * k2
        fn = lambda w: oracle.rd_rhs(w, D=kw["D"], bc=bc)  # noqa: E731
    else:
        sym = -1.0 * 1.0 * k2
        fn = lambda w: oracle.ac_rhs(w, bc=bc, **kw)  # noqa: E731
    return sym, fn, bc


@pytest.mark.parametrize("i", range(5))
def test_etd1_matches_reference(i):
    """ExponentialEuler: the phi1 table and three steps (fp32: identical torch ops)."""
    g = load_golden(f"etd1_{i}")
    dt = float(g["dt"])
    sym, fn, bc = etd1_case(g)
    # float32 exp of this host against the fixture's: an ulp or so on the table
    np.testing.assert_allclose(oracle.phi1(dt * sym).numpy(), g["phi1"], rtol=3e-7, atol=0)
    mult = oracle.etd1_multiplier(sym, dt)
    v = t32(g["u0"])
    for _ in range(3):
        v = oracle.imex_step(v, mult, fn, bc)
    assert oracle.rel_to_max(v.numpy(), g["u3"]) < 1e-6
    sym64, fn64, _ = etd1_case(g, torch.float64)
    np.testing.assert_allclose(oracle.phi1(dt * sym64).numpy(), g["phi1"], rtol=2e-6, atol=0)
    m64 = oracle.etd1_multiplier(sym64, dt)
    v = torch.tensor(g["u0"]).unsqueeze(0)
    for _ in range(3):
        v = oracle.imex_step(v, m64, fn64, bc)
    assert oracle.rel_to_max(v.numpy(), g["u3"]) < 1e-5


def test_ch_imex_fp64_matches_reference():
    g = load_golden("ch_imex_fp64")
    u0 = torch.tensor(g["u0"], dtype=torch.float64).unsqueeze(0)
    u = oracle.ch_imex_run(u0, int(g["n"]), 0.1)
    assert oracle.rel_to_max(u.numpy(), g["u"]) < 1e-13


def test_ch_grad_matches_reference_autograd():
    g = load_golden("ch_grad")
    c0 = torch.tensor(g["u0"], dtype=torch.float64).unsqueeze(0)
    tgt = torch.tensor(g["target"], dtype=torch.float64).unsqueeze(0)
    loss, g0, gD, ge = oracle.ch_imex_loss_grads(c0, tgt, int(g["n"]), float(g["dt"]),
                                                 float(g["eps"]), float(g["D"]))
    assert abs(loss - float(g["loss"])) <= 1e-14 * abs(float(g["loss"]))
    assert oracle.rel_to_max(g0.numpy(), g["g_c0"]) < 1e-12
    assert abs(gD - float(g["g_D"])) <= 1e-10 * abs(float(g["g_D"]))
    assert abs(ge - float(g["g_eps"])) <= 1e-10 * abs(float(g["g_eps"]))


def test_driver_run_matches_reference():
    g = load_golden("driver_ch")
    u = oracle.ch_imex_run(t32(g["u0"]), int(g["n"]), 0.1)
    assert oracle.rel_to_max(u.numpy()[0], g["c"]) < 1e-6


def test_vjp_is_consistent_with_loss_gradient():
    """One-step VJP of the oracle equals the autograd gradient of a 1-step loss."""
    shape = (6, 5, 7)
    u0 = torch.tensor(oracle.seeded_ch_field(shape, 3), dtype=torch.float64).unsqueeze(0)
    tgt = torch.tensor(oracle.seeded_ch_field(shape, 4), dtype=torch.float64).unsqueeze(0)
    loss, g0, gD, ge = oracle.ch_imex_loss_grads(u0, tgt, 1, 0.1, 2.0, 1.2)
    u1 = oracle.ch_imex_run(u0, 1, 0.1, 2.0, 1.2)
    lam = 2 * (u1 - tgt) / u1.numel()
    gu, vD, ve = oracle.ch_imex_vjp(u0, lam, 0.1, 2.0, 1.2)
    assert oracle.rel_to_max(gu.numpy(), g0.numpy()) < 1e-13
    assert abs(vD - gD) < 1e-12 * max(1.0, abs(gD))
    assert abs(ve - ge) < 1e-12 * max(1.0, abs(ge))


def test_normalize_bc_errors_match_reference_messages():
    with pytest.raises(ValueError, match="exactly three axis entries"):
        oracle.normalize_bc(("periodic", "periodic"))
    with pytest.raises(ValueError, match="require explicit values"):
        oracle.normalize_bc(("dirichlet", "periodic", "periodic"))
    with pytest.raises(ValueError, match="Unsupported BC type"):
        oracle.normalize_bc(("robin", "periodic", "periodic"))
    with pytest.raises(ValueError, match="two boundary values"):
        oracle.normalize_bc((("dirichlet", (1.0,)), "periodic", "periodic"))
    with pytest.raises(ValueError, match="do not accept boundary values"):
        oracle.normalize_bc((("neumann", (1.0, 2.0)), "periodic", "periodic"))


def test_steady_state_loop_semantics():
    """The steady-state loop (evoxels/solvers.py:218-247): with check_freq = 1 it stops at the first
    iteration whose relative change ||u - step(u)||_F / sqrt(Nx Ny Nz) is <= conv_crit, having applied
    the step that many times plus one; a larger check_freq checks only multiples of it; max_iters
    bounds a run that does not converge."""
    shape = (8, 6, 5)
    bc = (("dirichlet", (0.0, 0.0)), "neumann", "neumann")
    u0 = torch.tensor(oracle.seeded_unit_field(shape, 7), dtype=torch.float32).unsqueeze(0)

    def step(v):
        return oracle.fe_step(v, 0.15, lambda w: oracle.rd_rhs(w, 1.0, bc))
    crit = 1e-4
    u, it, conv, checks = oracle.steady_state_run(u0, step, 5000, crit, 1)
    assert conv and [c[0] for c in checks] == list(range(it))
    rel = [c[1][0] for c in checks]
    assert rel[-1] <= crit and all(r > crit for r in rel[:-1])
    ref = u0
    for _ in range(it):
        ref = step(ref)
    assert torch.equal(u, ref)
    _, it7, conv7, checks7 = oracle.steady_state_run(u0, step, 5000, crit, 7)
    assert conv7 and it7 >= it and (it7 - 1) % 7 == 0 and all(c[0] % 7 == 0 for c in checks7)
    _, itn, convn, _ = oracle.steady_state_run(u0, step, 23, 0.0, 5)
    assert not convn and itn == 23


def regular_solution_mu(c, lib):
    """The logarithmic bulk term of the reference's solver notebook."""
    return lib.log(c) - lib.log(1 - c) + 3.0 * (1 - 2 * c)


@pytest.mark.parametrize("i", range(2))
def test_ch_rhs_regular_solution_bitexact(i):
    g = load_golden(f"ch_log_rhs_{i}")
    r = oracle.ch_rhs(t32(g["u0"]), 3.0, 1.0, parse_bc(g["bc"]), mu_hom=regular_solution_mu)
    np.testing.assert_array_equal(r.numpy(), g["rhs"])


def test_driver_regular_solution_matches_reference():
    g = load_golden("driver_ch_log")
    u = oracle.ch_imex_run(t32(g["u0"]), int(g["n"]), 0.1, mu_hom=regular_solution_mu)
    assert oracle.rel_to_max(u.numpy()[0], g["c"]) < 1e-6

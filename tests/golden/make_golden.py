"""Generate the golden fixtures in this folder by running the evoxels reference.

Run where the reference is checked out, with its path in ``EVOXELS_REF`` (the
folder that holds the ``evoxels`` package; there is no default), and torch on
CPU::

    EVOXELS_REF=<path of the evoxels checkout> python tests/golden/make_golden.py [--only=name,name]

(``--only`` writes just the named fixtures.)

The reference package is imported with a small shim: ``matplotlib`` is absent
here, so stub modules stand in for it (only plotting uses it), and the package
``__init__`` is bypassed because it imports the JAX-only inversion module.
Everything that produces numbers below is the reference's own code:
``CahnHilliard.rhs``, ``ReactionDiffusion.rhs``, ``PseudoSpectralIMEX``,
``ForwardEuler``, ``CellCenteredBCs.pad_bc`` and ``run_cahn_hilliard_solver``,
all on ``device='cpu'``, ``jit=False``.

Each fixture is a small ``.npz`` (fields of at most 16^3 voxels).  Inputs are
the seeded float64 arrays the product and the oracle both consume.
"""

from __future__ import annotations

import os
import sys
import types
import warnings

import numpy as np
import torch

REF = os.environ.get("EVOXELS_REF", "")
OUT = os.path.dirname(os.path.abspath(__file__))


def import_reference():
    """Import the reference's torch-path modules without matplotlib/JAX."""
    if not REF or not os.path.isdir(os.path.join(REF, "evoxels")):
        raise SystemExit("set EVOXELS_REF to the folder holding the reference's evoxels package")
    for name in ("matplotlib", "matplotlib.pyplot", "matplotlib.widgets", "matplotlib.patches"):
        if name not in sys.modules:
            mod = types.ModuleType(name)
            sys.modules[name] = mod
    sys.modules["matplotlib.widgets"].Slider = object
    sys.modules["matplotlib.patches"].Patch = object
    sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]
    if "evoxels" not in sys.modules:
        pkg = types.ModuleType("evoxels")
        pkg.__path__ = [os.path.join(REF, "evoxels")]
        sys.modules["evoxels"] = pkg
    import importlib
    mods = {}
    for m in ("voxelfields", "voxelgrid", "problem_definition", "timesteppers",
              "solvers", "precompiled_solvers.cahn_hilliard"):
        mods[m] = importlib.import_module("evoxels." + m)
    return mods


def ch_field(shape, seed):
    rng = np.random.default_rng(seed)
    return 0.5 + 0.1 * rng.random(shape)


def unit_field(shape, seed):
    rng = np.random.default_rng(seed)
    return rng.random(shape)


def make_vg(R, shape, precision="float32", domain=None):
    vf = R["voxelfields"].VoxelFields(shape, domain_size=domain or shape)
    vf.precision = precision
    return vf, R["voxelgrid"].VoxelGridTorch(vf.grid_info(), precision=precision, device="cpu")


def main():
    R = import_reference()
    PD, TS = R["problem_definition"], R["timesteppers"]
    warnings.simplefilter("ignore")
    torch.set_default_dtype(torch.float32)
    out = {}

    # 1) the reference test's exact mixed-BC ghost golden (tests/test_solvers.py:105-126)
    _, vg = make_vg(R, (2, 2, 2), domain=(1, 1, 1))
    prob = PD.ReactionDiffusion(vg, D=1.0, bc=(("dirichlet", (10.0, 20.0)), "neumann", "periodic"))
    field = vg.init_scalar_field(np.arange(1, 9, dtype=np.float32).reshape(2, 2, 2))
    out["pad_mixed"] = dict(u=field.numpy(), padded=prob.pad_bc(field).numpy())

    # 2) CahnHilliard.rhs, fp32, periodic and non-periodic, odd shapes, clip exercised
    cases = [((8, 8, 8), 11, None, (1.0, 1.0, 1.0)),
             ((5, 7, 9), 12, None, (1.0, 1.0, 1.0)),
             ((12, 10, 6), 13, None, (0.5, 0.75, 1.25)),
             ((9, 8, 7), 14, (("dirichlet", (0.2, 0.7)), "neumann", "periodic"), (1.0, 1.0, 1.0)),
             ((6, 9, 8), 15, ("neumann", ("dirichlet", (0.0, 1.0)), "neumann"), (1.0, 1.0, 1.0))]
    for i, (shape, seed, bc, spacing) in enumerate(cases):
        domain = tuple(n * h for n, h in zip(shape, spacing))
        _, vg = make_vg(R, shape, domain=domain)
        u0 = ch_field(shape, seed)
        if i == 1:  # push some voxels outside [0, 1] so clip matters
            u0 = u0 + 0.8 * (unit_field(shape, 99) - 0.5)
        kw = dict(eps=3.0, D=1.0)
        if bc is not None:
            kw["bc"] = bc
        prob = PD.CahnHilliard(vg, **kw)
        u = vg.init_scalar_field(u0)
        r = prob.rhs(0.0, u)
        out[f"ch_rhs_{i}"] = dict(u0=u0, rhs=r.numpy(), shape=np.array(shape),
                                  spacing=np.array(spacing), bc=np.array(repr(bc)))

    # 3) PseudoSpectralIMEX on CahnHilliard: 1 step and 10 steps, fp32, plus eps/D variants
    for i, (shape, seed, eps, D, dt, n) in enumerate([((16, 16, 16), 21, 3.0, 1.0, 0.1, 1),
                                                       ((16, 16, 16), 21, 3.0, 1.0, 0.1, 10),
                                                       ((12, 10, 14), 22, 1.0, 0.7, 0.1, 10),
                                                       ((10, 12, 9), 23, 2.5, 1.6, 0.05, 5)]):
        _, vg = make_vg(R, shape)
        prob = PD.CahnHilliard(vg, eps=eps, D=D)
        st = TS.PseudoSpectralIMEX(prob, dt)
        u0 = ch_field(shape, seed)
        u = vg.init_scalar_field(u0)
        for _ in range(n):
            u = st.step(0.0, u)
        out[f"ch_imex_{i}"] = dict(u0=u0, u=u.numpy(), shape=np.array(shape), eps=eps, D=D, dt=dt, n=n)

    # 3b) PseudoSpectralIMEX with a non-periodic x axis (mirrored FFT extension)
    nx_cases = [((16, 12, 10), 24, ("neumann", "periodic", "periodic"), 3.0, 1.0, 0.1, 5),
                ((8, 16, 12), 25, (("dirichlet", (0.0, 0.0)), "periodic", "periodic"), 2.0, 1.2, 0.1, 5),
                ((10, 8, 9), 26, (("dirichlet", (0.2, 0.7)), "periodic", "periodic"), 3.0, 1.0, 0.05, 4),
                ((12, 10, 8), 27, ("neumann", "periodic", "periodic"), 1.5, 0.8, 0.1, 6)]
    for i, (shape, seed, bc, eps, D, dt, n) in enumerate(nx_cases):
        _, vg = make_vg(R, shape)
        prob = PD.CahnHilliard(vg, eps=eps, D=D, bc=bc)
        st = TS.PseudoSpectralIMEX(prob, dt)
        u0 = ch_field(shape, seed)
        u = vg.init_scalar_field(u0)
        for _ in range(n):
            u = st.step(0.0, u)
        out[f"ch_imex_nx_{i}"] = dict(u0=u0, u=u.numpy(), shape=np.array(shape), eps=eps, D=D, dt=dt, n=n,
                                      bc=np.array(repr(bc)))

    # 3c) TwoPhaseAllenCahn.rhs (19-point normal Laplacian, every BC kind, flat clipped
    #     regions for the |grad|^2 <= 1e-7 branch) and RungeKutta4 steps
    ac_cases = [((10, 9, 8), 41, None, dict()),
                ((8, 12, 10), 42, ("periodic", "periodic", "periodic"), dict(eps=3.0, curvature=0.2)),
                ((9, 8, 11), 43, (("dirichlet", (0.0, 1.0)), "neumann", "periodic"),
                 dict(eps=1.5, gab=0.7, M=1.3, force=0.4, curvature=0.05)),
                ((7, 10, 9), 44, ("periodic", ("dirichlet", (0.2, 0.9)), ("dirichlet", (1.0, 0.0))),
                 dict(eps=2.5, curvature=0.5))]
    ac_cases.append(((12, 10, 8), 45, None, dict(curvature=0.1)))   # blocky: flat clipped halves
    for i, (shape, seed, bc, kw) in enumerate(ac_cases):
        _, vg = make_vg(R, shape)
        if bc is not None:
            kw = dict(kw, bc=bc)
        prob = PD.TwoPhaseAllenCahn(vg, **kw)
        u0 = 1.4 * unit_field(shape, seed) - 0.2
        if i == 4:   # two flat half-spaces (|grad|^2 = 0) with a noisy slab between them
            u0 = np.where(np.arange(shape[0])[:, None, None] < shape[0] // 2, 1.3, -0.2) + 0 * u0
            u0[5:7] = unit_field((2,) + shape[1:], seed)
        u = vg.init_scalar_field(u0)
        r = prob.rhs(0.0, u)
        st = TS.RungeKutta4(prob, 0.1)
        v = u
        for _ in range(3):
            v = st.step(0.0, v)
        out[f"ac_{i}"] = dict(u0=u0, rhs=r.numpy(), u3=v.numpy(), shape=np.array(shape), bc=np.array(repr(bc)),
                              kw=np.array(repr(kw)))

    # 3d) RKC1 / RKC2 steps over three problems' rhs; the float32 stage coefficients
    #     are stored too (libm may round cosh/arccosh differently on another host)
    rkc_cases = [("RKC1", "TwoPhaseAllenCahn", (10, 9, 8), 61, None, dict(), 0.1, {}),
                 ("RKC2", "TwoPhaseAllenCahn", (8, 12, 10), 62, (("dirichlet", (0.0, 1.0)), "neumann", "periodic"),
                  dict(eps=1.5, curvature=0.05), 0.2, {}),
                 ("RKC1", "ReactionDiffusion", (9, 8, 7), 63, ("neumann", "periodic", ("dirichlet", (1.0, 0.0))),
                  dict(D=1.0), 0.05, dict(polygrad=7, damping=0.1)),
                 ("RKC2", "ReactionDiffusion", (8, 8, 8), 64, None, dict(D=0.8), 0.2, dict(polygrad=6)),
                 ("RKC2", "CahnHilliard", (8, 10, 12), 65, None, dict(eps=3.0, D=1.0), 0.01, {})]
    for i, (scheme, pname, shape, seed, bc, kw, dt, skw) in enumerate(rkc_cases):
        _, vg = make_vg(R, shape)
        if bc is not None:
            kw = dict(kw, bc=bc)
        prob = getattr(PD, pname)(vg, **kw)
        u0 = (1.4 * unit_field(shape, seed) - 0.2) if pname != "CahnHilliard" else ch_field(shape, seed)
        st = getattr(TS, scheme)(prob, dt, **skw)
        u = vg.init_scalar_field(u0)
        for _ in range(3):
            u = st.step(0.0, u)
        co = {k: getattr(st, k).numpy() for k in ("mu0", "mu1", "mu11", "nu", "c", "gamma") if hasattr(st, k)}
        out[f"rkc_{i}"] = dict(u0=u0, u3=u.numpy(), shape=np.array(shape), bc=np.array(repr(bc)), kw=np.array(repr(kw)),
                               scheme=np.array(scheme), problem=np.array(pname), dt=dt, skw=np.array(repr(skw)),
                               **co)

    # 3e) ExponentialEuler (ETD1, Pade phi1) steps: periodic and mirrored x, power-of-two
    #     and other nx, three problems; the phi1 table is stored too
    etd_cases = [("CahnHilliard", (8, 10, 12), 71, None, dict(eps=3.0, D=1.0), 0.05),
                 ("CahnHilliard", (12, 8, 10), 72, ("neumann", "periodic", "periodic"), dict(eps=2.0, D=0.7), 0.1),
                 ("ReactionDiffusion", (10, 8, 8), 73, (("dirichlet", (0.2, 1.0)), "periodic", "periodic"),
                  dict(D=1.0), 0.5),
                 ("TwoPhaseAllenCahn", (8, 8, 12), 74, ("periodic", "periodic", "periodic"), dict(eps=2.0), 0.3),
                 ("CahnHilliard", (16, 12, 10), 75, (("dirichlet", (0.0, 1.0)), "periodic", "periodic"),
                  dict(eps=3.0, D=1.0), 0.1)]
    for i, (pname, shape, seed, bc, kw, dt) in enumerate(etd_cases):
        _, vg = make_vg(R, shape)
        if bc is not None:
            kw = dict(kw, bc=bc)
        prob = getattr(PD, pname)(vg, **kw)
        u0 = ch_field(shape, seed) if pname == "CahnHilliard" else unit_field(shape, seed)
        st = TS.ExponentialEuler(prob, dt)
        u = vg.init_scalar_field(u0)
        for _ in range(3):
            u = st.step(0.0, u)
        out[f"etd1_{i}"] = dict(u0=u0, u3=u.numpy(), shape=np.array(shape), bc=np.array(repr(bc)),
                                kw=np.array(repr(kw)), problem=np.array(pname), dt=dt,
                                phi1=st.phi_1_k_squared.numpy())

    # 4) true FP64 CH IMEX (default dtype float64 so the k-grid is fp64 too)
    torch.set_default_dtype(torch.float64)
    shape = (16, 16, 16)
    _, vg = make_vg(R, shape, precision="float64")
    prob = PD.CahnHilliard(vg)
    st = TS.PseudoSpectralIMEX(prob, 0.1)
    u0 = ch_field(shape, 21)
    u = vg.init_scalar_field(u0)
    for _ in range(10):
        u = st.step(0.0, u)
    out["ch_imex_fp64"] = dict(u0=u0, u=u.numpy(), n=10)
    torch.set_default_dtype(torch.float32)

    # 5) ReactionDiffusion + ForwardEuler (the explicit FD path), generic and specialised pads
    fd_cases = [((9, 8, 7), 31, (("dirichlet", (0, 0)), "neumann", "neumann"), 1.0 / 60, 10),
                ((8, 8, 8), 32, None, 1.0 / 60, 10),
                ((7, 9, 10), 33, (("dirichlet", (10.0, 20.0)), "neumann", "periodic"), 1.0 / 60, 5),
                ((10, 6, 8), 34, ("neumann", "periodic", "periodic"), 1.0 / 60, 5),
                ((6, 8, 12), 35, (("dirichlet", (1.0, -1.0)), "periodic", "periodic"), 1.0 / 60, 5)]
    for i, (shape, seed, bc, dt, n) in enumerate(fd_cases):
        _, vg = make_vg(R, shape)
        kw = dict(D=1.0)
        if bc is not None:
            kw["bc"] = bc
        prob = PD.ReactionDiffusion(vg, **kw)
        st = TS.ForwardEuler(prob, dt)
        u0 = unit_field(shape, seed)
        u = vg.init_scalar_field(u0)
        for _ in range(n):
            u = st.step(0.0, u)
        out[f"fd_fe_{i}"] = dict(u0=u0, u=u.numpy(), shape=np.array(shape), bc=np.array(repr(bc)),
                                 dt=dt, n=n)

    # 6) torch autograd through the reference: dL/dc0, dL/dD, dL/deps, fp64
    torch.set_default_dtype(torch.float64)
    shape = (8, 8, 8)
    _, vg = make_vg(R, shape, precision="float64")
    u0 = ch_field(shape, 41)
    tgt = ch_field(shape, 42)
    Dt = torch.tensor(1.3, requires_grad=True)
    et = torch.tensor(2.0, requires_grad=True)
    prob = PD.CahnHilliard(vg, eps=et, D=Dt)
    st = TS.PseudoSpectralIMEX(prob, 0.1)
    c0 = vg.init_scalar_field(u0).requires_grad_(True)
    u = c0
    for _ in range(5):
        u = st.step(0.0, u)
    loss = torch.mean((u - vg.init_scalar_field(tgt)) ** 2)
    loss.backward()
    out["ch_grad"] = dict(u0=u0, target=tgt, n=5, D=1.3, eps=2.0, dt=0.1, loss=float(loss),
                          g_c0=c0.grad.numpy(), g_D=float(Dt.grad), g_eps=float(et.grad))
    torch.set_default_dtype(torch.float32)

    # 7) the drop-in driver end to end: run_cahn_hilliard_solver on CPU, fp32
    vf = R["voxelfields"].VoxelFields((16, 16, 16), domain_size=(16, 16, 16))
    u0 = ch_field((16, 16, 16), 51)
    vf.add_field("c", u0.copy())
    R["precompiled_solvers.cahn_hilliard"].run_cahn_hilliard_solver(
        vf, "c", "torch", jit=False, device="cpu", time_increment=0.1, frames=2, max_iters=20,
        verbose=False)
    out["driver_ch"] = dict(u0=u0, c=vf.fields["c"], n=20)

    # 8) the regular-solution (logarithmic) bulk term of the reference's solver notebook
    #    (docs/notebooks/01-using-solvers.ipynb): CahnHilliard.rhs and the drop-in driver
    def regular_solution_mu(c, lib):
        return lib.log(c) - lib.log(1 - c) + 3.0 * (1 - 2 * c)
    for i, (shape, seed, bc) in enumerate([((12, 10, 16), 61, None),
                                           ((9, 8, 12), 62, ("neumann", "periodic", "periodic"))]):
        _, vg = make_vg(R, shape)
        kw = dict(eps=3.0, D=1.0, mu_hom=regular_solution_mu)
        if bc is not None:
            kw["bc"] = bc
        prob = PD.CahnHilliard(vg, **kw)
        u0 = ch_field(shape, seed)
        r = prob.rhs(0.0, vg.init_scalar_field(u0))
        out[f"ch_log_rhs_{i}"] = dict(u0=u0, rhs=r.numpy(), shape=np.array(shape), bc=np.array(repr(bc)))
    vf = R["voxelfields"].VoxelFields((16, 16, 16), domain_size=(16, 16, 16))
    u0 = ch_field((16, 16, 16), 63)
    vf.add_field("c", u0.copy())
    R["precompiled_solvers.cahn_hilliard"].run_cahn_hilliard_solver(
        vf, "c", "torch", jit=False, device="cpu", time_increment=0.1, frames=2, max_iters=20,
        eps=3.0, diffusivity=1.0, mu_hom=regular_solution_mu, verbose=False)
    out["driver_ch_log"] = dict(u0=u0, c=vf.fields["c"], n=20)

    only = [a.split("=", 1)[1].split(",") for a in sys.argv[1:] if a.startswith("--only=")]
    for name, arrays in out.items():
        if only and name not in only[0]:
            continue
        np.savez_compressed(os.path.join(OUT, name + ".npz"), **arrays)
    print("wrote", len(only[0]) if only else len(out), "fixtures to", OUT)


if __name__ == "__main__":
    main()

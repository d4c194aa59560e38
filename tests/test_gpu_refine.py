"""GPU parity of the model refinement (ModelBase/ModelRefiner.cpp) and of the
coarse-grid objective built on it (Inversion/ThreeDModelObjective.h:254-260,
310-324) against the oracle.

Tolerances: projection and combination are copies and ordered FP64 sums, so
they must agree bit for bit (signed zeros included); the forward and gradient on the
refined grid are the FP64 path (relative norm error <= 1e-10).
"""
import dataclasses

import numpy as np
import pytest

from helpers import oracle_forward, oracle_lqderivative, relerr, small_survey
from jif3d_gb300 import capi, workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-10


def same_bits(a, b):
    """Bit-for-bit equality (np.array_equal does not tell -0.0 from +0.0)."""
    a, b = np.ascontiguousarray(a, dtype=np.float64), np.ascontiguousarray(b, dtype=np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.int64), b.view(np.int64))


def refine(s, refs):
    """The refined survey of coarse survey ``s`` (same stations, background,
    kind), its axes refined at ``refs`` as ModelRefiner::RefineAxes does."""
    fs = [capi.refine_axis(s.coords(a), (s.xsize, s.ysize, s.zsize)[a], refs[a])
          for a in range(3)]
    return dataclasses.replace(s, xsize=fs[0], ysize=fs[1], zsize=fs[2])


def coarse_sizes(s):
    return [s.xsize, s.ysize, s.zsize]


def fine_setup(ctx, coarse, fine):
    W.setup_context(ctx, fine)
    ctx.set_refinement(*coarse_sizes(coarse))


def oracle_project(O, coarse, fine, cvec, nblock, nextra, fvec=None):
    cg, fg = coarse.ngrid, fine.ngrid
    out = np.zeros(nblock * fg + nextra) if fvec is None else np.array(fvec, dtype=float)
    for b in range(nblock):
        prev = None if fvec is None else out[b * fg:(b + 1) * fg]
        out[b * fg:(b + 1) * fg] = O.refine_project(coarse_sizes(coarse), coarse_sizes(fine),
                                                    cvec[b * cg:(b + 1) * cg], prev)
    out[nblock * fg:] = cvec[nblock * cg:]
    return out


def oracle_combine(O, coarse, fine, fvec, nblock, nextra):
    cg, fg = coarse.ngrid, fine.ngrid
    out = np.zeros(nblock * cg + nextra)
    for b in range(nblock):
        out[b * cg:(b + 1) * cg] = O.refine_combine(coarse_sizes(coarse), coarse_sizes(fine),
                                                    fvec[b * fg:(b + 1) * fg])
    out[nblock * cg:] = fvec[nblock * fg:]
    return out


def random_refs(rng, s, per_axis=(9, 8, 7)):
    refs = []
    for a in range(3):
        c = s.coords(a)
        r = rng.uniform(c[0], c[-1], per_axis[a]).round(1)
        r = np.unique(np.concatenate([r, c[rng.integers(0, c.size, 2)]]))
        refs.append(r)
    return refs


def test_reference_refiner_case_on_device(ctx, oracle_lib):
    """test_ModelRefiner.cpp:115-147 on the device: iota projected, a unit
    gradient combined to 60 on every coarse cell."""
    s = small_survey(W.SCALAR, seed=1, bg=False, origin=(0.0, 0.0, 0.0))
    s = dataclasses.replace(s, xsize=np.full(2, 50.0), ysize=np.full(3, 40.0),
                            zsize=np.full(5, 30.0), model=np.arange(30.0))
    f = refine(s, [10.0 * np.arange(20), 20.0 * np.arange(20), 5.0 * np.arange(50)])
    assert f.shape == (10, 6, 30)
    fine_setup(ctx, s, f)
    info = ctx.refinement_info()
    assert info == dict(coarse_cells=30, coarse_nparm=30, covers_all=True)
    fine = ctx.refine_project(s.model)
    assert same_bits(fine, oracle_project(oracle_lib, s, f, s.model, 1, 0))
    assert np.all(ctx.refine_combine(np.ones(f.ngrid)) == 60.0)


@pytest.mark.parametrize("kind,nmodels", [(W.SCALAR, 1), (W.SCALAR, 3), (W.TENSOR, 2),
                                          (W.MAGNETIZATION, 2)])
def test_project_combine_bit_exact(ctx, oracle_lib, kind, nmodels):
    """Irregular coarse cells, refinement coordinates that repeat coarse
    corners, background parameters (copied) or three magnetisation blocks;
    device and host forms against the oracle, bit for bit."""
    import torch
    s = small_survey(kind, seed=20 + kind, nx=6, ny=5, nz=4, bg=kind != W.MAGNETIZATION)
    rng = np.random.default_rng(kind * 10 + nmodels)
    s.xsize = s.xsize + rng.uniform(0, 1, s.xsize.size).round(2)
    f = refine(s, random_refs(rng, s))
    fine_setup(ctx, s, f)
    nblock = 3 if kind == W.MAGNETIZATION else 1
    nextra = 0 if kind == W.MAGNETIZATION else s.bg_thick.size
    cnp = nblock * s.ngrid + nextra
    assert ctx.refinement_info()["coarse_nparm"] == cnp
    assert ctx.sizes()["nparm"] == nblock * f.ngrid + nextra
    C = rng.normal(size=(nmodels, cnp))
    Fg = rng.normal(size=(nmodels, nblock * f.ngrid + nextra))
    refF = np.stack([oracle_project(oracle_lib, s, f, C[i], nblock, nextra)
                     for i in range(nmodels)])
    refC = np.stack([oracle_combine(oracle_lib, s, f, Fg[i], nblock, nextra)
                     for i in range(nmodels)])
    assert same_bits(ctx.refine_project(C), refF)
    assert same_bits(ctx.refine_combine(Fg), refC)
    dC, dF = torch.tensor(C, device="cuda"), torch.zeros(refF.shape, dtype=torch.float64,
                                                         device="cuda")
    ctx.refine_project_device(nmodels, dC.data_ptr(), dF.data_ptr())
    dG, dOut = torch.tensor(Fg, device="cuda"), torch.zeros_like(dC)
    ctx.refine_combine_device(nmodels, dG.data_ptr(), dOut.data_ptr())
    ctx.synchronize()
    assert same_bits(dF.cpu().numpy(), refF)
    assert same_bits(dOut.cpu().numpy(), refC)


def test_uncovered_cells_keep_values(ctx, oracle_lib):
    """A forward mesh wider than the coarse grid: refined cells outside every
    coarse run keep the values they had (device and host forms); their
    gradient entries do not reach the coarse gradient."""
    import torch
    s = small_survey(W.SCALAR, seed=31, nx=2, ny=2, nz=1, bg=False, origin=(0.0, 0.0, 0.0))
    s = dataclasses.replace(s, xsize=np.array([10.0]), ysize=np.array([4.0, 6.0]),
                            zsize=np.array([5.0]), model=np.array([1.0, 2.0]))
    f = dataclasses.replace(s, xsize=np.array([5.0, 5.0, 5.0]), ysize=np.array([2.0, 2.0, 6.0]),
                            zsize=np.array([5.0]))
    fine_setup(ctx, s, f)
    assert not ctx.refinement_info()["covers_all"]
    prev = np.full(9, -7.0)
    ref = oracle_project(oracle_lib, s, f, s.model, 1, 0, prev)
    assert same_bits(ctx.refine_project(s.model, prev), ref)
    dF = torch.full((9,), -7.0, dtype=torch.float64, device="cuda")
    dC = torch.tensor(s.model, device="cuda")
    ctx.refine_project_device(1, dC.data_ptr(), dF.data_ptr())
    ctx.synchronize()
    assert same_bits(dF.cpu().numpy(), ref)
    g = np.arange(9.0)
    assert same_bits(ctx.refine_combine(g), oracle_combine(oracle_lib, s, f, g, 1, 0))


@pytest.mark.parametrize("kind", [W.SCALAR, W.TENSOR, W.MAGNETIC])
def test_coarse_objective_through_refinement(ctx, oracle_lib, kind):
    """ImplDataDifference / ImplGradient with a fine model geometry: data of
    the projected model on the refined grid, coarse gradient = combined fine
    gradient with the background entries passed through; against the oracle
    on the refined survey, and against central differences of the coarse
    objective."""
    s = small_survey(kind, seed=40 + kind, nx=4, ny=4, nz=3, nmeas=7)
    rng = np.random.default_rng(kind)
    f = refine(s, random_refs(rng, s, (6, 5, 5)))
    fine_setup(ctx, s, f)
    fmodel = ctx.refine_project(s.model)
    d = ctx.forward(fmodel)
    dref = oracle_forward(oracle_lib, f, fmodel)
    assert relerr(d, dref) <= TOL
    misfit = rng.normal(size=d.size) * np.abs(d).mean()  # residuals at the data's scale
    gfine = ctx.lqderivative(fmodel, misfit)
    gc = ctx.refine_combine(gfine)
    gref = oracle_combine(oracle_lib, s, f, oracle_lqderivative(oracle_lib, f, misfit, fmodel),
                          1, s.bg_thick.size)
    assert relerr(gc, gref) <= TOL
    # the coarse objective phi(c) = |F(P c) - obs|^2 with obs = F(P c0) - misfit,
    # whose gradient at c0 is P^T 2 J^T misfit
    obs = d - misfit

    def phi(c):
        r = ctx.forward(ctx.refine_project(c)) - obs
        return float(r @ r)
    for i in (0, s.ngrid // 2, s.ngrid - 1, s.ngrid):  # three cells and a background layer
        h = 1e-3 * max(1.0, abs(s.model[i]))
        cp, cm = s.model.copy(), s.model.copy()
        cp[i] += h
        cm[i] -= h
        fd = (phi(cp) - phi(cm)) / (2 * h)
        assert abs(fd - gc[i]) <= 1e-6 * max(abs(fd), abs(gc[i])) + 1e-12, (i, fd, gc[i])


def test_refinement_state_and_errors(ctx):
    s = small_survey(W.SCALAR, seed=50)
    W.setup_context(ctx, s)
    with pytest.raises(capi.J3GError):  # the mesh change cleared any refinement
        ctx.refine_project(np.zeros(s.nparm))
    ctx.set_refinement(*coarse_sizes(s))
    assert ctx.refinement_info()["coarse_nparm"] == s.nparm
    # the identity refinement: projection and combination are copies
    assert same_bits(ctx.refine_project(s.model), s.model)
    assert same_bits(ctx.refine_combine(s.model), s.model)
    W.setup_context(ctx, s)
    with pytest.raises(capi.J3GError):
        ctx.refinement_info()
    with pytest.raises(capi.J3GError):
        ctx.set_refinement(np.zeros(0), s.ysize, s.zsize)


def test_large_refinement_adjoint_identity(ctx, oracle_lib):
    """64 x 64 x 32 coarse cells refined 2 x 2 x 2 (about 1 M refined cells),
    two models: bit-exact against the oracle, and <P c, f> = <c, P^T f>."""
    import torch
    xs = np.full(64, 50.0)
    zs = np.array([25.0 * 1.05 ** k for k in range(32)])
    s = W.Survey("coarse", xs, xs.copy(), zs, (0.0, 0.0, 0.0), np.zeros((1, 3)), W.SCALAR,
                 np.zeros(64 * 64 * 32))
    # the fine model's corners, the end of the domain last (not used, as in
    # the reference)
    refs = [np.arange(129) * 25.0, np.arange(129) * 25.0,
            np.sort(np.concatenate([s.coords(2), s.coords(2)[:-1] + 0.5 * zs]))]
    f = refine(s, refs)
    assert f.shape == (128, 128, 64)
    fine_setup(ctx, s, f)
    rng = np.random.default_rng(5)
    C = rng.normal(size=(2, s.ngrid))
    Fg = rng.normal(size=(2, f.ngrid))
    dC, dF = torch.tensor(C, device="cuda"), torch.zeros((2, f.ngrid), dtype=torch.float64,
                                                         device="cuda")
    dG, dOut = torch.tensor(Fg, device="cuda"), torch.zeros_like(dC)
    ctx.refine_project_device(2, dC.data_ptr(), dF.data_ptr())
    ctx.refine_combine_device(2, dG.data_ptr(), dOut.data_ptr())
    ctx.synchronize()
    PF, PtG = dF.cpu().numpy(), dOut.cpu().numpy()
    assert same_bits(PF[1], oracle_project(oracle_lib, s, f, C[1], 1, 0))
    assert same_bits(PtG[0], oracle_combine(oracle_lib, s, f, Fg[0], 1, 0))
    for i in range(2):
        lhs, rhs = float(PF[i] @ Fg[i]), float(C[i] @ PtG[i])
        assert abs(lhs - rhs) <= 1e-12 * np.linalg.norm(PF[i]) * np.linalg.norm(Fg[i])


@pytest.mark.parametrize("case", ["long_rows", "odd_rows", "long_runs"])
def test_kernel_paths(ctx, oracle_lib, case):
    """The kernels' launch variants against the oracle, bit for bit: rows of
    more than 64 refined z cells and more than 32 coarse z cells (lanes loop
    over chunks), odd row lengths (no paired stores), z runs longer than 4
    (the run-length loop)."""
    import torch
    zs = {"long_rows": np.full(40, 8.0), "odd_rows": np.array([5.0, 7.0, 9.0]),
          "long_runs": np.array([12.0, 20.0])}[case]
    s = small_survey(W.SCALAR, seed=60, nx=3, ny=2, nz=zs.size, bg=False,
                     origin=(0.0, 0.0, 0.0))
    s = dataclasses.replace(s, zsize=zs, model=np.zeros(3 * 2 * zs.size))
    zc = s.coords(2)
    zref = {"long_rows": np.sort(np.concatenate([zc, zc[:-1] + 4.0])),
            "odd_rows": np.array([0.0, 2.0, 5.0, 7.0, 9.0, 12.0, 15.0, 21.0]),
            "long_runs": np.arange(0.0, 33.0, 2.0)}[case]
    f = refine(s, [s.coords(0), s.coords(1), zref])
    expect_fnz = {"long_rows": 80, "odd_rows": 7, "long_runs": 16}[case]
    assert f.zsize.size == expect_fnz
    fine_setup(ctx, s, f)
    rng = np.random.default_rng(61)
    C = rng.normal(size=(2, s.ngrid))
    Fg = rng.normal(size=(2, f.ngrid))
    # signed zeros: a sum that starts with -0.0 (or holds only zeros) must
    # come out as the reference's 0.0 + ... does
    Fg[:, ::7] = -0.0
    Fg[1, : 2 * f.zsize.size] = -0.0
    dC, dF = torch.tensor(C, device="cuda"), torch.zeros((2, f.ngrid), dtype=torch.float64,
                                                         device="cuda")
    dG, dOut = torch.tensor(Fg, device="cuda"), torch.zeros_like(dC)
    ctx.refine_project_device(2, dC.data_ptr(), dF.data_ptr())
    ctx.refine_combine_device(2, dG.data_ptr(), dOut.data_ptr())
    ctx.synchronize()
    for i in range(2):
        assert same_bits(dF[i].cpu().numpy(), oracle_project(oracle_lib, s, f, C[i], 1, 0))
        assert same_bits(dOut[i].cpu().numpy(), oracle_combine(oracle_lib, s, f, Fg[i], 1, 0))


def test_cpp_refiner(oracle_lib, tmp_path):
    """jif3D::GB300ModelRefiner (the C++ drop-in for ModelRefiner) driven as
    ThreeDModelObjective drives its refiner: refined axes, projected values
    and combined gradient against the oracle, bit for bit; a copied refiner
    gives the same gradient; a zero-size last cell throws FatalException."""
    import os
    import subprocess
    from jif3d_gb300 import build as B
    B.build()
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    exe = str(tmp_path / "refiner_check")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(root, "include"),
                        "-I", os.path.join(root, "jif3d_gb300", "host"),
                        os.path.join(here, "cpp", "refiner_check.cpp"),
                        "-L", os.path.dirname(B.LIB), "-ljif3d_gb300",
                        "-Wl,-rpath," + os.path.dirname(B.LIB), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    O = oracle_lib
    rng = np.random.default_rng(70)
    cs = [rng.integers(10, 30, 5).astype(float) + 0.25, rng.integers(10, 30, 4).astype(float),
          rng.integers(5, 20, 6) * 1.1]
    origin = (-3.0, 2.5, 0.0)
    cc = [O.corners(o, c) for o, c in zip(origin, cs)]
    refs = [np.sort(rng.uniform(c[0], c[-1], 9).round(1)) for c in cc]
    fs = [O.refine_axis(c, s_, r_) for c, s_, r_ in zip(cc, cs, refs)]
    values = rng.normal(size=int(np.prod([c.size for c in cs])))
    fgrad = rng.normal(size=int(np.prod([f.size for f in fs])))
    fgrad[::5] = -0.0
    with open(tmp_path / "p.txt", "w") as f:
        parts = [repr(float(v)) for v in origin]
        for v in (*cs, *refs, values, fgrad):
            parts += [str(len(v))] + [repr(float(x)) for x in v]
        f.write(" ".join(parts))
    r = subprocess.run([exe, str(tmp_path / "p.txt"), str(tmp_path / "o.txt")],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out, exc = {}, False
    for line in open(tmp_path / "o.txt"):
        p = line.split()
        if p[:2] == ["exception", "ok"]:
            exc = True
            continue
        out[p[0]] = np.array([float(v) for v in p[2:]])
    for a, name in enumerate(("xsizes", "ysizes", "zsizes")):
        assert same_bits(out[name], fs[a])
    assert same_bits(out["fine"], O.refine_project(cs, fs, values))
    ref_grad = O.refine_combine(cs, fs, fgrad)
    assert same_bits(out["coarse_grad"], ref_grad)
    assert same_bits(out["copy_grad"], ref_grad)
    assert exc

"""Residual VJPs as the adjoint drivers use them.

* torch.autograd.Function backward == explicit VJP kernels;
* directional derivatives of the residual against central finite
  differences over 32 seeded directions in the control m and the state u
  (a scheme whose own error is far below the gate: h = 1 in u, where R is
  affine, Richardson-extrapolated h = 1e-2 / 5e-3 in m) — the accuracy gate
  is 1e-6 relative, met at the 512x512 inverse-problem configuration by the
  FP32-quadrature and FP64 VJPs alike;
* the reduced gradient of J(m) = 0.5 |u(m) - d|^2 against femx's own
  ReducedFunctional (femx/inverse/ReducedFunctional.hpp:94-117) run on the
  reference library with DenseLinearSolver (tests/golden/inverse_12.npz).
  Linear solves here use scipy on the host: they are test infrastructure,
  the assembly, Dirichlet rows and VJPs run on the GPU.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from conftest import load_golden, rel_inf  # noqa: E402
from femx_gb300 import assembly as A  # noqa: E402
from femx_gb300 import meshes  # noqa: E402
from femx_gb300.autograd import p1_kappa_residual  # noqa: E402
from oracle import pyoracle as orc  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from femx_gb300 import build
    build.build()


def dev(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    return (t if dtype is None else t.to(dtype)).cuda()


def setup(nx, seed, jitter=True):
    coords, conn = meshes.jittered_tri(nx, seed=seed) if jitter else meshes.structured_tri(nx)
    offs, dofs = meshes.scalar_elem_dofs(conn)
    n, e = coords.shape[0], conn.shape[0]
    amap = A.makeAssemblyMap(n, n, dev(offs), dev(dofs), dev(offs), dev(dofs))
    bdofs = meshes.dirichlet_dofs(coords, meshes.boundary_nodes(coords))
    bc = A.makeBoundaryMap(dev(bdofs), amap.pattern())
    return coords, conn, amap, bc, bdofs


class OracleResidual:
    """R(u, m) with Dirichlet rows replaced, from the serial CPU oracle.

    Central differences need two residuals whose rounding errors are
    correlated; the GPU's FP64 L2 reductions sum in a run-dependent order,
    and that noise divided by 2h would swamp small directional derivatives.
    The oracle evaluates the same operator in a fixed order."""

    def __init__(self, coords, conn, f, bdofs, g):
        offs, dofs = meshes.scalar_elem_dofs(conn)
        n = coords.shape[0]
        self.m = orc.AssemblyMap(n, n, offs, dofs, offs, dofs)
        self.q = orc.P1Quad(coords, conn)
        self.b = orc.BoundaryMap(bdofs, self.m.row_ptr, self.m.col_ind)
        self.f, self.g = f, g

    def __call__(self, u, mvec):
        r, _ = orc.assemble_p1_kappa(self.m, self.q, np.exp(mvec), self.f, u)
        return self.b.replace_res(u, self.g, r)


def test_autograd_backward_equals_vjp_kernels():
    coords, conn, amap, bc, bdofs = setup(20, 1)
    rng = np.random.default_rng(1)
    n, e = coords.shape[0], conn.shape[0]
    u = dev(rng.standard_normal(n)).requires_grad_()
    m = dev(0.5 * rng.standard_normal(e)).requires_grad_()
    lam = dev(rng.standard_normal(n))
    g = dev(rng.standard_normal(len(bdofs)))
    r = p1_kappa_residual(u, m, amap, dev(coords), dev(meshes.fourier_source(coords, 2)), bc, g)
    (r * lam).sum().backward()
    lam_t = lam.clone()
    lam_t[dev(bdofs).long()] = 0.0
    gu = torch.zeros(n, dtype=torch.float64, device="cuda")
    gm = torch.zeros(e, dtype=torch.float64, device="cuda")
    A.vjpP1Kappa(amap, dev(coords), torch.exp(m.detach()), u.detach(), lam_t, gu, gm)
    gu[dev(bdofs).long()] += lam[dev(bdofs).long()]
    # FP64 reductions at L2 sum in a run-dependent order: equal to rounding
    assert rel_inf(u.grad.cpu().numpy(), gu.cpu().numpy()) <= 1e-14
    assert rel_inf(m.grad.cpu().numpy(), gm.cpu().numpy()) <= 1e-14


def directional_fd(R, u0, m0, lam, d, which):
    """Central differences of lam^T R along a unit direction, with a scheme
    whose own error is far below the 1e-6 gate. R is affine in u, so one
    central difference with h = 1 is exact up to rounding; in m it is smooth
    (kappa = exp(m)), so two central differences (h = 1e-2 and 5e-3) are
    combined by Richardson extrapolation, removing the h^2 term."""
    if which == "u":
        return float((R(u0 + d, m0) - R(u0 - d, m0)) @ lam) / 2.0

    def central(h):
        return float((R(u0, m0 + h * d) - R(u0, m0 - h * d)) @ lam) / (2 * h)
    return (4.0 * central(5e-3) - central(1e-2)) / 3.0


# Jittered mesh: the FP32-quadrature element carries the FP32 rounding of its
# geometry (~1e-7 per element), which a directional derivative over many
# elements can amplify, hence its looser gate there. On a uniform mesh the
# FP32 geometry is exact and the gradient reduction runs in FP64, so the
# FP32-quadrature gradient meets 1e-6 (test_config4_vjp_512 below).
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-8), ("mixed", 1e-8), ("fp32_quad", 1e-4)])
def test_vjp_matches_central_differences_32_directions(precision, tol):
    coords, conn, amap, bc, bdofs = setup(64, 4)
    rng = np.random.default_rng(4)
    n, e = coords.shape[0], conn.shape[0]
    f = meshes.fourier_source(coords, 1)
    m0 = meshes.grf_centroids(coords, conn, seed=4, ell=0.05, grid=128)
    u0 = rng.standard_normal(n)
    g = np.zeros(len(bdofs))
    lam = rng.standard_normal(n)
    u = dev(u0).requires_grad_()
    m = dev(m0).requires_grad_()
    r = p1_kappa_residual(u, m, amap, dev(coords), dev(f), bc, dev(g), precision=precision)
    (r * dev(lam)).sum().backward()
    gu, gm = u.grad.cpu().numpy(), m.grad.cpu().numpy()
    R = OracleResidual(coords, conn, f, bdofs, g)
    errs = []
    for _ in range(32):
        dm = rng.standard_normal(e)
        dm /= np.linalg.norm(dm)
        fd = directional_fd(R, u0, m0, lam, dm, "m")
        errs.append(abs(fd - gm @ dm) / abs(fd))
        du = rng.standard_normal(n)
        du /= np.linalg.norm(du)
        fd = directional_fd(R, u0, m0, lam, du, "u")
        errs.append(abs(fd - gu @ du) / abs(fd))
    assert max(errs) <= tol, max(errs)


@pytest.mark.parametrize("precision", ["fp32_quad", "fp64"])
def test_config4_vjp_512(precision):
    """The inverse-problem configuration: 512x512 uniform mesh, m = log kappa
    a seeded GRF (correlation length 0.05, variance 1), Dirichlet rows. The
    state and control VJPs (behind torch.autograd.Function) along 32 seeded
    unit directions each, against the oracle's exact gradient, and against
    central differences of the oracle's FP64 residual on 8 of them; gate
    1e-6 relative, for the FP32-quadrature mode too."""
    coords, conn, amap, bc, bdofs = setup(512, 4, jitter=False)
    rng = np.random.default_rng(4)
    n, e = coords.shape[0], conn.shape[0]
    f = meshes.fourier_source(coords, 1)
    m0 = meshes.grf_centroids(coords, conn, seed=4, ell=0.05, var=1.0, grid=512)
    u0 = rng.standard_normal(n)
    lam = rng.standard_normal(n)
    g = np.zeros(len(bdofs))
    u = dev(u0).requires_grad_()
    m = dev(m0).requires_grad_()
    r = p1_kappa_residual(u, m, amap, dev(coords), dev(f), bc, dev(g), precision=precision)
    (r * dev(lam)).sum().backward()
    gu, gm = u.grad.cpu().numpy(), m.grad.cpu().numpy()
    # the oracle's exact gradient (zeroBoundary on lam, lam on the constrained rows)
    offs, dofs = meshes.scalar_elem_dofs(conn)
    om = orc.AssemblyMap(n, n, offs, dofs, offs, dofs)
    oq = orc.P1Quad(coords, conn)
    lt = lam.copy()
    lt[bdofs] = 0.0
    ogu, ogm = orc.vjp_p1_kappa(om, oq, np.exp(m0), u0, lt)
    ogu[bdofs] += lam[bdofs]
    R = OracleResidual(coords, conn, f, bdofs, g)
    exact, fd_errs = [], []
    for i in range(32):
        dm = rng.standard_normal(e)
        dm /= np.linalg.norm(dm)
        du = rng.standard_normal(n)
        du /= np.linalg.norm(du)
        exact.append(abs((gm - ogm) @ dm) / abs(ogm @ dm))
        exact.append(abs((gu - ogu) @ du) / abs(ogu @ du))
        if i < 8:
            fd = directional_fd(R, u0, m0, lam, dm, "m")
            fd_errs.append(abs(fd - gm @ dm) / abs(fd))
            fd = directional_fd(R, u0, m0, lam, du, "u")
            fd_errs.append(abs(fd - gu @ du) / abs(fd))
    assert max(exact) <= 1e-6, max(exact)
    assert max(fd_errs) <= 1e-6, max(fd_errs)


def test_gradcheck_small():
    coords, conn, amap, bc, bdofs = setup(5, 2)
    rng = np.random.default_rng(2)
    n, e = coords.shape[0], conn.shape[0]
    u = dev(rng.standard_normal(n)).requires_grad_()
    m = dev(0.3 * rng.standard_normal(e)).requires_grad_()
    coords_d, f_d = dev(coords), dev(meshes.fourier_source(coords, 3))
    g = dev(rng.standard_normal(len(bdofs)))
    assert torch.autograd.gradcheck(
        lambda uu, mm: p1_kappa_residual(uu, mm, amap, coords_d, f_d, bc, g), (u, m),
        eps=1e-6, atol=1e-8, rtol=1e-6, nondet_tol=1e-12)


def test_reduced_gradient_matches_femx_reduced_functional():
    import scipy.sparse.linalg as spla
    gd = load_golden("inverse_12")
    coords, conn = gd["coords"], gd["conn"]
    offs, dofs = meshes.scalar_elem_dofs(conn)
    n, e = coords.shape[0], conn.shape[0]
    amap = A.makeAssemblyMap(n, n, dev(offs), dev(dofs), dev(offs), dev(dofs))
    bdofs = meshes.dirichlet_dofs(coords, meshes.boundary_nodes(coords))
    bc = A.makeBoundaryMap(dev(bdofs), amap.pattern())
    coords_d, f_d = dev(coords), dev(gd["f"])
    m = dev(gd["m"])
    g = dev(np.zeros(len(bdofs)))
    zero = torch.zeros(n, dtype=torch.float64, device="cuda")
    # LinearStateSolver (femx/state/StateSolver.hpp:90-108): rhs = -R(0),
    # J = dR/du with constrained rows replaced, solve.
    r0 = p1_kappa_residual(zero, m, amap, coords_d, f_d, bc, g).detach()
    jac = A.CsrMatrix(amap.pattern())
    res = torch.empty(n, dtype=torch.float64, device="cuda")
    A.assembleP1Kappa(amap, coords_d, torch.exp(m), f_d, zero, res, jac)
    A.replaceRows(bc, jac, 1.0)
    J = jac.to_scipy()
    u = spla.spsolve(J.tocsc(), -r0.cpu().numpy())
    assert rel_inf(u, gd["u"]) <= 1e-10
    value = 0.5 * float(np.sum((u - gd["d"]) ** 2))
    assert abs(value - float(gd["value"][0])) <= 1e-10 * abs(float(gd["value"][0]))
    # adjoint: J^T lam = dJ/du; grad = dJ/dm - (dR/dm)^T lam
    lam = spla.spsolve(J.T.tocsc(), u - gd["d"])
    u_t = dev(u).requires_grad_()
    m_t = m.clone().requires_grad_()
    r = p1_kappa_residual(u_t, m_t, amap, coords_d, f_d, bc, g)
    (r * dev(lam)).sum().backward()
    grad = -m_t.grad.cpu().numpy()
    assert rel_inf(grad, gd["grad"]) <= 1e-9


# ------------------------------------------------ Taylor-Hood autograd

def th_setup(nx, seed):
    c3, k3 = meshes.jittered_tri(nx, seed=seed)
    cp2, conn6, nv = meshes.p2_mesh(c3, k3)
    offs, dofs, nd = meshes.th_elem_dofs(conn6, cp2.shape[0])
    amap = A.makeAssemblyMap(nd, nd, dev(offs), dev(dofs), dev(offs), dev(dofs))
    bd, bv = meshes.cavity_dirichlet(cp2, cp2.shape[0])
    bc = A.makeBoundaryMap(dev(bd), amap.pattern())
    return cp2, conn6, nv, nd, offs, dofs, amap, bd, bv, bc


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32_quad", 1e-6)])
def test_taylor_hood_autograd_backward_is_the_transpose_action(precision, tol):
    """backward() of the constrained Taylor-Hood residual against the
    oracle's Jacobian transposed: g = J~^T lam with the constrained rows of
    J~ replaced by identity rows (what replaceRes makes of R); and the
    viscosity derivative against the oracle's residuals at nu = 1 and 0."""
    from femx_gb300.autograd import taylor_hood_residual
    cp2, conn6, nv, nd, offs, dofs, amap, bd, bv, bc = th_setup(6, 12)
    state = meshes.cavity_state(cp2, nv, seed=12)
    lam = np.random.default_rng(12).standard_normal(nd)
    s = dev(state).requires_grad_()
    nu = torch.tensor(2e-2, dtype=torch.float64, device="cuda", requires_grad=True)
    r = taylor_hood_residual(s, nu, amap, dev(cp2), dev(conn6, torch.int32), bc, dev(bv),
                             precision=precision)
    (r * dev(lam)).sum().backward()
    om = orc.AssemblyMap(nd, nd, offs, dofs, offs, dofs)
    _, vals = orc.assemble_th_ns(om, cp2, conn6, 2e-2, state)
    vals = orc.BoundaryMap(bd, om.row_ptr, om.col_ind).replace_rows(vals, 1.0)
    g_ref = orc.matvec_t(om.row_ptr, om.col_ind, vals, lam, nd)
    assert rel_inf(s.grad.cpu().numpy(), g_ref) <= tol
    r1, _ = orc.assemble_th_ns(om, cp2, conn6, 1.0, state)
    r0, _ = orc.assemble_th_ns(om, cp2, conn6, 0.0, state)
    lt = lam.copy()
    lt[bd] = 0.0
    gnu = float(lt @ (r1 - r0))
    assert abs(float(nu.grad) - gnu) <= tol * abs(gnu)


def test_taylor_hood_gradcheck_small():
    from femx_gb300.autograd import taylor_hood_residual
    cp2, conn6, nv, nd, offs, dofs, amap, bd, bv, bc = th_setup(2, 3)
    s = dev(meshes.cavity_state(cp2, nv, seed=3)).requires_grad_()
    nu = torch.tensor(0.1, dtype=torch.float64, device="cuda", requires_grad=True)
    coords_d, c6 = dev(cp2), dev(conn6, torch.int32)
    g = dev(bv)
    assert torch.autograd.gradcheck(
        lambda ss, nn: taylor_hood_residual(ss, nn, amap, coords_d, c6, bc, g), (s, nu),
        eps=1e-6, atol=1e-8, rtol=1e-6, nondet_tol=1e-12)


@pytest.mark.parametrize("precision", ["fp64", "double_float"])
def test_tiled_autograd_gradcheck_and_reproducible(precision):
    """The tiled residual and VJPs behind the autograd function: gradcheck
    against its own finite differences (with no atomics the forward is
    deterministic, so nondet_tol is 0), backward bitwise equal over runs,
    and equal to the atomic FP64 path's gradients to rounding."""
    coords, conn, amap, bc, bdofs = setup(6, 4)
    rng = np.random.default_rng(4)
    n, e = coords.shape[0], conn.shape[0]
    coords_d, f_d = dev(coords), dev(meshes.fourier_source(coords, 3))
    amap.enableTiles(coords_d)
    g = dev(rng.standard_normal(len(bdofs)))
    u0, m0 = rng.standard_normal(n), 0.3 * rng.standard_normal(e)
    u = dev(u0).requires_grad_()
    m = dev(m0).requires_grad_()
    # double-float inputs keep 47 bits (a relative 2^-46 truncation), so its
    # central differences need a larger step: R is affine in u and smooth in m
    eps, atol = (1e-6, 1e-8) if precision == "fp64" else (1e-4, 1e-7)
    assert torch.autograd.gradcheck(
        lambda uu, mm: p1_kappa_residual(uu, mm, amap, coords_d, f_d, bc, g,
                                         precision=precision, tiled=True), (u, m),
        eps=eps, atol=atol, rtol=1e-6, nondet_tol=0.0)
    lam = dev(rng.standard_normal(n))
    grads = []
    for tiled in (True, True, False):
        uu, mm = dev(u0).requires_grad_(), dev(m0).requires_grad_()
        r = p1_kappa_residual(uu, mm, amap, coords_d, f_d, bc, g,
                              precision=precision if tiled else "fp64", tiled=tiled)
        (r * lam).sum().backward()
        grads.append((uu.grad.cpu().numpy(), mm.grad.cpu().numpy()))
    assert np.array_equal(grads[0][0], grads[1][0]) and np.array_equal(grads[0][1], grads[1][1])
    assert rel_inf(grads[0][0], grads[2][0]) <= 1e-13
    assert rel_inf(grads[0][1], grads[2][1]) <= 1e-13

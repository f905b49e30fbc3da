"""The GPU Taylor-Hood operator (gbfem_assemble_th_ns, through the C ABI)
pinned by the weak form itself, in every precision mode and in the
deterministic mode: exact integrals for linear fields on jittered meshes
(every row of R and J), exact and forced quadratic solutions (Poiseuille,
Couette, shear, stagnation flow, a pressure gradient) and the Jacobian's
identities (tests/th_checks.py). These pins share no code with the oracle.

Tolerances: FP64 and double-float 1e-12; FP32 quadrature 1e-6 (J and R);
MIXED J 1e-6 and R 1e-12 (its residual is computed to FP64 accuracy). For
linear fields the diffusion terms cancel in the interior rows, so R is much
smaller than its terms: the FP32 and double-float residuals (about 24 and 48
significant bits) are measured against the size of the terms there.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

import th_checks as T  # noqa: E402
import th_exact as X  # noqa: E402
from femx_gb300 import assembly as A  # noqa: E402
from femx_gb300 import meshes  # noqa: E402

MODES = [
    # precision, deterministic, tol_r, tol_j
    ("fp64", False, 1e-12, 1e-12),
    ("fp64", True, 1e-12, 1e-12),
    ("fp32_quad", False, 1e-6, 1e-6),
    ("fp32_quad", True, 1e-6, 1e-6),
    ("mixed", False, 1e-12, 1e-6),
    ("mixed", True, 1e-12, 1e-6),
    ("double_float", False, 1e-12, 1e-12),
    ("double_float", True, 1e-12, 1e-12),
]
IDS = [f"{p}{'-det' if d else ''}" for p, d, _, _ in MODES]


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from femx_gb300 import build
    build.build()


def gpu_assembler(precision, deterministic):
    def run(cp2, conn6, nd, nu, state):
        offs, dofs, _ = meshes.th_elem_dofs(conn6, cp2.shape[0])
        d = lambda a, t=None: torch.from_numpy(np.ascontiguousarray(a)).cuda() if t is None \
            else torch.from_numpy(np.ascontiguousarray(a)).to(t).cuda()
        m = A.makeAssemblyMap(nd, nd, d(offs, torch.int32), d(dofs, torch.int32),
                              d(offs, torch.int32), d(dofs, torch.int32))
        res = torch.zeros(nd, dtype=torch.float64, device="cuda")
        jac = A.CsrMatrix(m.pattern())
        A.assembleTaylorHood(m, d(cp2), d(conn6, torch.int32), nu, d(state), res, jac,
                             precision=precision, deterministic=deterministic)
        m.check()
        torch.cuda.synchronize()
        p = m.pattern()
        return (res.cpu().numpy(),
                X.dense(p.row_ptr.cpu().numpy(), p.col_ind.cpu().numpy(),
                        jac.vals.cpu().numpy(), nd))
    return run


@pytest.mark.parametrize("precision,det,tol_r,tol_j", MODES, ids=IDS)
def test_linear_fields_match_exact_integrals(precision, det, tol_r, tol_j):
    # FP32 and double-float round relative to the size of R's terms, which
    # cancel for these fields (R is much smaller than its terms); FP64 and
    # MIXED (FP64-accurate residual) are held to ||R||_inf itself
    T.check_linear_fields(gpu_assembler(precision, det), tol_r, tol_j,
                          r_scale="terms" if precision in ("fp32_quad", "double_float")
                          else "ref")


@pytest.mark.parametrize("precision,det,tol_r,tol_j", MODES, ids=IDS)
def test_patch_solutions(precision, det, tol_r, tol_j):
    T.check_patch_solutions(gpu_assembler(precision, det), tol_r)


@pytest.mark.parametrize("precision,det,tol_r,tol_j", MODES, ids=IDS)
def test_jacobian_identities(precision, det, tol_r, tol_j):
    T.check_jacobian_identities(gpu_assembler(precision, det), tol_j)

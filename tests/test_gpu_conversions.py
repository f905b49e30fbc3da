"""The FP32 element paths convert between double and float with integer bit
operations (the hardware conversion issues on GB300's FP64 pipe). These must
agree bit for bit with IEEE-754 round-to-nearest-even conversion."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from femx_gb300 import build
    build.build()


def run_probe(values: np.ndarray):
    from femx_gb300 import _lib
    x = torch.from_numpy(np.ascontiguousarray(values, dtype=np.float64)).cuda()
    f = torch.empty(x.numel(), dtype=torch.float32, device="cuda")
    d = torch.empty(x.numel(), dtype=torch.float64, device="cuda")
    _lib.check(_lib.lib().gbfem_probe_convert(
        x.numel(), C.c_void_p(x.data_ptr()), C.c_void_p(f.data_ptr()), C.c_void_p(d.data_ptr()),
        C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    torch.cuda.synchronize()
    return x, f, d


def test_conversions_match_ieee_round_to_nearest_even():
    rng = np.random.default_rng(0)
    parts = [
        rng.standard_normal(1 << 20),
        rng.standard_normal(1 << 18) * 10.0 ** rng.integers(-40, 40, size=1 << 18),
        np.array([0.0, -0.0, 1.0, -1.0, 3.4028234663852886e38, 3.4028235677973366e38,
                  1.1754943508222875e-38, 1.401298464324817e-45, 5e-324, np.inf, -np.inf,
                  1e300, -1e-300]),
    ]
    # halfway cases: doubles exactly between two floats (ties to even), and
    # values one ulp either side of the tie
    base = rng.standard_normal(1 << 16).astype(np.float32).astype(np.float64)
    ulp = np.spacing(base.astype(np.float32)).astype(np.float64)
    tie = base + 0.5 * ulp
    parts += [tie, np.nextafter(tie, np.inf), np.nextafter(tie, -np.inf)]
    vals = np.concatenate(parts)
    x, f, d = run_probe(vals)
    ref_f = x.to(torch.float32)
    assert torch.equal(f.view(torch.int32), ref_f.view(torch.int32))
    assert torch.equal(d, ref_f.to(torch.float64))


def test_nan_stays_nan():
    _, f, d = run_probe(np.array([np.nan, -np.nan]))
    assert torch.isnan(f).all() and torch.isnan(d).all()


def test_scatter_conversion_is_exact_except_subnormals():
    from femx_gb300 import _lib
    rng = np.random.default_rng(1)
    specials = np.array([0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan,
                         3.4028234663852886e38, -3.4028234663852886e38,
                         1.1754943508222875e-38, -1.1754943508222875e-38,   # smallest normals
                         1.1754942106924411e-38, 1.401298464324817e-45,     # subnormals
                         -1.401298464324817e-45], dtype=np.float32)
    bits = rng.integers(0, 1 << 32, size=1 << 20, dtype=np.uint64).astype(np.uint32)
    vals = np.concatenate([specials, bits.view(np.float32),
                           rng.standard_normal(1 << 18).astype(np.float32)])
    x = torch.from_numpy(vals).cuda()
    out = torch.empty(x.numel(), dtype=torch.float64, device="cuda")
    _lib.check(_lib.lib().gbfem_probe_convert_ftz(
        x.numel(), C.c_void_p(x.data_ptr()), C.c_void_p(out.data_ptr()),
        C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    torch.cuda.synchronize()
    ref = x.to(torch.float64)
    sub = (x != 0) & (x.abs() < 1.1754943508222875e-38)
    ref = torch.where(sub, torch.copysign(torch.zeros_like(ref), ref), ref)
    nan = torch.isnan(ref)
    assert torch.equal(torch.isnan(out), nan)
    assert torch.equal(out[~nan].view(torch.int64), ref[~nan].view(torch.int64))
    assert int(sub.sum()) > 0


def test_newton_reciprocal_is_within_two_ulps():
    from femx_gb300 import _lib
    rng = np.random.default_rng(4)
    x = np.concatenate([rng.standard_normal(1 << 18) * 10.0 ** rng.integers(-35, 35, size=1 << 18),
                        np.array([1.0, -1.0, 3.0, 1e-30, -1e30, 2.0 ** -120, 2.0 ** 120,
                                  2.0 ** -121, 2.0 ** 122, 1e-300, 1e300, 5e-324])])
    xd = torch.from_numpy(x).cuda()
    out = torch.empty_like(xd)
    _lib.check(_lib.lib().gbfem_probe_rcp(xd.numel(), C.c_void_p(xd.data_ptr()),
                                          C.c_void_p(out.data_ptr()), 0,
                                          C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    with np.errstate(over="ignore", divide="ignore"):
        ref = 1.0 / x
    fin = np.isfinite(ref) & (ref != 0)
    ulp = np.abs(got[fin] - ref[fin]) / np.spacing(np.abs(ref[fin]))
    assert ulp.max() <= 2.0
    assert np.array_equal(got[~fin], ref[~fin])


def test_newton_reciprocal_square_root_is_within_two_ulps():
    from femx_gb300 import _lib
    rng = np.random.default_rng(5)
    x = np.concatenate([np.abs(rng.standard_normal(1 << 18)) * 10.0 ** rng.integers(-35, 35, size=1 << 18),
                        np.array([1.0, 4.0, 2.0, 1e-30, 1e30, 2.0 ** -120, 2.0 ** 120,
                                  2.0 ** -121, 2.0 ** 122, 1e-300, 1e300, 0.0, -1.0])])
    xd = torch.from_numpy(x).cuda()
    out = torch.empty_like(xd)
    _lib.check(_lib.lib().gbfem_probe_rcp(xd.numel(), C.c_void_p(xd.data_ptr()),
                                          C.c_void_p(out.data_ptr()), 1,
                                          C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    with np.errstate(divide="ignore", invalid="ignore"):
        ref = 1.0 / np.sqrt(x)
    fin = np.isfinite(ref) & (ref != 0)
    ulp = np.abs(got[fin] - ref[fin]) / np.spacing(np.abs(ref[fin]))
    assert ulp.max() <= 2.0
    assert np.isinf(got[x == 0.0]).all() and np.isnan(got[x < 0]).all()

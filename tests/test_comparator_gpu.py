"""The timing comparator (the reference's GPU force kernel restated in
comparator/ref_nbody.cu) computes what the
reference's kernel computes: forces against the FP64 oracle at FP32
accuracy, Force.w = sum_j (r^-12 - r^-6), the virial sum W/6 and the
clamped r^2 RDF over all ordered pairs."""
import ctypes as C
import os

import numpy as np
import pytest

import lj_testutil as U

pytestmark = pytest.mark.gpu


def _lib():
    import comparator
    return comparator.load()


@pytest.mark.parametrize("n,block", [(2000, 256), (1000, 128), (300, 512)])
def test_reference_kernel_restatement(ljgb_mod, oracle_mod, n, block):
    torch = pytest.importorskip("torch")
    rho = 0.8
    pos, _, L = U.lattice_state(n, rho, 1.0, "fcc", 0.03, seed=n)
    lib = _lib()
    p4 = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    p4[:, :3] = torch.from_numpy(pos.astype(np.float32)).cuda()
    f4 = torch.zeros_like(p4)
    scratch = torch.zeros(int(lib.ljref_scratch_bytes(n, block)) // 4 + 4, dtype=torch.int32, device="cuda")
    dr2 = float(ljgb_mod.reference_rdf_dr2(n))
    st = torch.cuda.current_stream().cuda_stream
    assert lib.ljref_forces(p4.data_ptr(), f4.data_ptr(), n, L, 1, dr2, block, scratch.data_ptr(), st) == 0
    rdf = np.zeros(256, np.int32)
    press = C.c_float()
    assert lib.ljref_results(scratch.data_ptr(), n, block, rdf.ctypes.data, C.byref(press), st) == 0
    f = f4.cpu().numpy().astype(np.float64)
    # FP64 oracle on the same float positions
    p32 = pos.astype(np.float32).astype(np.float64)
    r = oracle_mod.f64_forces(p32, L, True)
    err = U.force_errors(f[:, :3], r["F"])
    assert err["gate_max"] < 2e-4, err          # FP32 arithmetic, plain sums
    # Force.w = sum_j (r^-12 - r^-6) = e_i / 4 (unscaled)
    assert np.allclose(f[:, 3], r["e"] / 4.0, rtol=1e-4, atol=1e-4 * np.abs(r["e"]).max())
    # pressure word: sum_i 4/6 sum_j s r^2 = W / 6
    assert press.value == pytest.approx(r["W"] / 6.0, rel=1e-4)
    # every ordered pair is binned once (the last bin collects r^2 beyond it)
    assert int(rdf.sum()) == n * (n - 1)
    d = p32[:, None, :] - p32[None, :, :]
    d -= L * np.round(d / L)
    d2 = (d * d).sum(-1)[~np.eye(n, dtype=bool)]
    want = np.bincount(np.minimum((d2 / dr2).astype(np.int64), 255), minlength=256)
    assert np.abs(rdf - want).sum() <= 1e-4 * n * n    # float vs double binning at bin edges

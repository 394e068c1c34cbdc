"""The exact adjoint of the Born modelling operator (sfwi_born_adjoint).

L maps a model perturbation m = (dVp, dVs) to the scattered records of a
stage-2 forward run (sfwi_gpu_buffer_m + sfwi_run_forward); sfwi_born_adjoint
applies L^T to records.  The dot-product test pins the pair:

    <L m, d> = <m, L^T d>

on a 60x30 model with PML 10 and 250 steps, two shots (one over the whole
model, one over a 36-node window whose edge columns collect the PML cells
cut from them), so the split-field PML update, the window edges, the Born
region and the receivers all enter.  Both sides run in FP32 with FP64 sums:
with d = L m (no cancellation) the two sides agree within 1e-5 relative;
with random data within 1e-4 of |L m| |d| (the Cauchy-Schwarz scale).  The
adjoint is linear and additive over shots: L^T of a batch is the sum of the
shots' L^T (to the rounding of the FP64 sums), and L^T (2 d) = 2 L^T d.
The Gauss-Newton Hessian-vector product sfwi_hessian_vector is L^T L m:
the same bits as the adjoint of the forward records, symmetric
(<m2, H m1> = <H m2, m1>) and <m, H m> = |L m|^2, both within 1e-5.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ALLNX, ALLNZ, PML, NT, DX, DT, F0 = 60, 30, 10, 250, 10.0, 1e-3, 25.0


@pytest.fixture(scope="module")
def setup():
    from sfwi_gb300 import synth
    vp, vs, _ = synth.layered_model(ALLNX, ALLNZ, DX, vmin=1800.0, vmax=3000.0)
    vp0 = synth.smooth_z(vp, 3)
    vs0 = (vp0 / 1.73).astype(np.float32)
    full = synth.shot_descriptor(int(24 * DX), (np.arange(0, ALLNX) * DX).astype(np.int64), DX, PML, 0, sy=2, gy=0)
    win = synth.shot_descriptor(int(40 * DX), (np.arange(22, 58) * DX).astype(np.int64), DX, PML, 0, sy=3, gy=1)
    rng = np.random.default_rng(17)
    m = ((rng.standard_normal((ALLNX, ALLNZ)) * 40.0).astype(np.float32),
         (rng.standard_normal((ALLNX, ALLNZ)) * 25.0).astype(np.float32))
    return dict(vp0=vp0, vs0=vs0, shots=[full, win], m=m, sou=synth.ricker(NT, DT, F0))


def _engine(s):
    import sfwi_gb300 as sg
    fd = sg.FD2DGPU_ELASTIC(s["sou"], DX, DX, DT, ALLNX + 2 * PML, ALLNZ + 2 * PML, ALLNX, ALLNZ, 1, PML, NT, 4, 0,
                            stage=2)
    fd.GPUbufferVPVS(s["vp0"], s["vs0"])
    return fd


def _enqueue(fd, d, rz=None, rx=None):
    fd.enqueue_shot(d["nx"], d["isx"], d["isz"], d["igz"], d["ngx_left"], d["delta_left"], 0, d["gc"], rz, rx)


def _forward(s, m, shots):
    """L m: the scattered records of each shot, float32"""
    fd = _engine(s)
    fd.GPUbufferM(*m)
    for d in shots:
        _enqueue(fd, d)
    fd.run_forward()
    out = []
    for i, d in enumerate(shots):
        r = fd.read_records(i, d["ntr"])
        out.append((r["syn_z"].copy(), r["syn_x"].copy()))
    fd.close()
    return out


def _adjoint(s, data, shots):
    fd = _engine(s)
    for d, (rz, rx) in zip(shots, data):
        _enqueue(fd, d, rz, rx)
    out = fd.born_adjoint()
    fd.close()
    return out


def _dot_records(a, b):
    return sum(float(np.dot(x.astype(np.float64).ravel(), y.astype(np.float64).ravel()))
               for p, q in zip(a, b) for x, y in zip(p, q))


def _dot_model(m, img):
    return float(np.dot(m[0].astype(np.float64).ravel(), img[0].ravel()) +
                 np.dot(m[1].astype(np.float64).ravel(), img[1].ravel()))


def test_dot_product_with_d_equal_to_l_m(setup):
    s = setup
    lm = _forward(s, s["m"], s["shots"])
    lhs = _dot_records(lm, lm)
    assert lhs > 0
    rhs = _dot_model(s["m"], _adjoint(s, lm, s["shots"]))
    print("<Lm, Lm> = %.9e, <m, L^T L m> = %.9e, rel %.2e" % (lhs, rhs, abs(lhs - rhs) / lhs))
    assert abs(lhs - rhs) <= 1e-5 * lhs


def test_dot_product_with_random_data(setup):
    s = setup
    rng = np.random.default_rng(23)
    lm = _forward(s, s["m"], s["shots"])
    d = [((rng.standard_normal(z.shape)).astype(np.float32), (rng.standard_normal(x.shape)).astype(np.float32))
         for z, x in lm]
    lhs = _dot_records(lm, d)
    rhs = _dot_model(s["m"], _adjoint(s, d, s["shots"]))
    scale = np.sqrt(_dot_records(lm, lm) * _dot_records(d, d))
    print("<Lm, d> = %.9e, <m, L^T d> = %.9e, |diff| / (|Lm||d|) %.2e" % (lhs, rhs, abs(lhs - rhs) / scale))
    assert abs(lhs - rhs) <= 1e-4 * scale


def test_adjoint_is_additive_over_shots_and_linear(setup):
    s = setup
    rng = np.random.default_rng(29)
    d = [((rng.standard_normal((sh["ntr"], NT))).astype(np.float32),
          (rng.standard_normal((sh["ntr"], NT))).astype(np.float32)) for sh in s["shots"]]
    both = _adjoint(s, d, s["shots"])
    one = [_adjoint(s, [d[k]], [s["shots"][k]]) for k in range(2)]
    for j in range(2):
        # the same terms; an edge model cell sums its window cells shot by shot
        assert np.allclose(both[j], one[0][j] + one[1][j], rtol=1e-12, atol=1e-12 * np.abs(both[j]).max())
        assert np.abs(one[1][j]).max() > 0
    twice = _adjoint(s, [(2 * z, 2 * x) for z, x in d], s["shots"])
    for j in range(2):
        assert np.allclose(twice[j], 2 * both[j], rtol=1e-6, atol=1e-6 * np.abs(both[j]).max())


def _hessian(s, m, shots):
    fd = _engine(s)
    for d in shots:
        _enqueue(fd, d)
    out = fd.hessian_vector(*m)
    fd.close()
    return out


def test_hessian_vector_is_the_adjoint_of_the_forward_records(setup):
    s = setup
    hv = _hessian(s, s["m"], s["shots"])
    ref = _adjoint(s, _forward(s, s["m"], s["shots"]), s["shots"])
    for a, b in zip(hv, ref):
        assert np.array_equal(a, b)
    assert np.abs(hv[0]).max() > 0


def test_hessian_vector_is_symmetric_and_positive(setup):
    s = setup
    rng = np.random.default_rng(31)
    m2 = ((rng.standard_normal((ALLNX, ALLNZ)) * 30.0).astype(np.float32),
          (rng.standard_normal((ALLNX, ALLNZ)) * 20.0).astype(np.float32))
    h1 = _hessian(s, s["m"], s["shots"])
    h2 = _hessian(s, m2, s["shots"])
    a, b = _dot_model(m2, h1), _dot_model(s["m"], h2)
    scale = np.sqrt(_dot_model(s["m"], h1) * _dot_model(m2, h2))
    print("<m2, H m1> = %.9e, <H m2, m1> = %.9e, rel %.2e" % (a, b, abs(a - b) / scale))
    assert abs(a - b) <= 1e-5 * scale
    lm = _forward(s, s["m"], s["shots"])
    q = _dot_model(s["m"], h1)
    assert q > 0
    assert abs(q - _dot_records(lm, lm)) <= 1e-5 * q

"""FFBP image formation (FFBP.m + FFBP_POLAR_NFFT.m, knabNFFT branch, with
BP_POLAR_NFFT.m / NFFT1_1D.m leaves) on the GPU against the oracle's
restatement of the same recursion (oracle/ffbp.py, FP64).

Scenario: the reference's synthetic point-target set-up
(BP_FBP_FFBP_main.m:7-103) scaled down -- 8 pulses, 64 frequency samples,
a 32 x 32 scene -- at two geometries where every level's regridding is one
the reference's NFFT1_2D can run.  Tolerances: FP64 rel-L2 <= 1e-9 over the
finite pixels with identical NaN (extrapolated) pixels; FP32 data
(coordinates and phases in FP64) rel-L2 <= 1e-5.  A geometry the reference
cannot run (an odd NFFT grid at the top level) is refused with
NFFT2D_ERR_INVALID_ARG, where the oracle refuses too.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCENES = {"R2km_step8cm": dict(R=2e3, step=0.08), "R10km_step10cm": dict(R=10e3, step=0.1)}


def _scene(name):
    from oracle import ffbp as F
    return F.point_target_scene(Np=8, nf=64, Nx=32, targets=((0.0, 0.0), (0.48, -0.64)), **SCENES[name])


@pytest.fixture(scope="module")
def oracle_images(orc):
    from oracle import ffbp as F
    out = {}
    for name in SCENES:
        data, sar = _scene(name)
        out[name] = F.ffbp(data, sar, 1, 8)
    return out


def _compare(got, want):
    nan_g, nan_w = np.isnan(got), np.isnan(want)
    assert np.array_equal(nan_g, nan_w)
    m = ~nan_w
    assert m.sum() > 0.9 * m.size
    return float(np.linalg.norm(got[m] - want[m]) / np.linalg.norm(want[m]))


@pytest.mark.parametrize("name", list(SCENES))
@pytest.mark.parametrize("prec,tol", [("f64", 1e-9), ("f32", 1e-5)])
def test_ffbp_matches_oracle(oracle_images, name, prec, tol):
    from miscellaneous_gb300.sar import FFBP
    data, sar = _scene(name)
    im = FFBP(data, 1, 8, c=sar["c"], fc=sar["fc"], BW=sar["BW"], f2=sar["f2"], precision=prec).cpu().numpy()
    err = _compare(im.astype(np.complex128), oracle_images[name])
    print(f"{name} {prec}: rel-L2 {err:.2e}")
    assert err <= tol


def test_ffbp_focuses_point_targets():
    """Physics: both point targets are focused at their pixels -- the image's
    two strongest local peaks sit there, well above the sidelobes."""
    from miscellaneous_gb300.sar import FFBP
    data, sar = _scene("R2km_step8cm")
    im = np.abs(FFBP(data, 1, 8, c=sar["c"], fc=sar["fc"], BW=sar["BW"], f2=sar["f2"]).cpu().numpy())
    im = np.nan_to_num(im)
    v = data["x_mat"][0]  # the scene axis (x along columns, y along rows)

    def near(px, py):
        r, c = int(np.argmin(np.abs(v - py))), int(np.argmin(np.abs(v - px)))
        return im[max(r - 1, 0):r + 2, max(c - 1, 0):c + 2].max()

    top = im.max()
    assert near(0.0, 0.0) > 0.8 * top and near(0.48, -0.64) > 0.8 * top
    # far from both targets the image is far below the peaks
    assert im[-4:, :4].max() < 0.3 * top


def test_ffbp_refuses_what_the_reference_cannot_run(orc):
    from miscellaneous_gb300 import _lib
    from miscellaneous_gb300.sar import FFBP
    from oracle import ffbp as F
    data, sar = F.point_target_scene(Np=16, nf=64, Nx=32, R=2e3, step=0.08)
    with pytest.raises(ValueError):
        F.ffbp(data, sar, 1, 16)
    with pytest.raises(_lib.NFFT2DError) as e:
        FFBP(data, 1, 16, c=sar["c"], fc=sar["fc"], BW=sar["BW"], f2=sar["f2"], precision="f64")
    assert e.value.status == _lib.ERR_INVALID_ARG

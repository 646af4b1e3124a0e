"""The reference test-suite's statistical acceptance protocols on the CUDA path,
through the public API (GaussMLEFitter / fit / ROIBatch) and the C ABI."""
import ctypes as C

import numpy as np
import pytest

import gaussmle_gb300 as G
import statistics_cases as SC

pytestmark = pytest.mark.gpu


def gpu_fit_api(model, box, camera, psf, data, xc, yc, maps, cons):
    """fit() as a user calls it: PSF in microns (pixel size 0.1 um)."""
    if model == 0:
        psf_um = G.GaussianXYNB(psf.sigma * 0.1)
    elif model == 3:  # widths in microns; gamma, d and z are in microns already
        psf_um = G.AstigmaticXYZNB(psf.sx0 * 0.1, psf.sy0 * 0.1, psf.Ax, psf.Ay, psf.Bx,
                                   psf.By, psf.gamma, psf.d)
    else:
        psf_um = psf
    fitter = G.GaussMLEFitter(psf_model=psf_um, constraints=cons)
    if camera == 0:
        res = G.fit(fitter, data)
    else:
        var, gain, off = maps
        cam = G.SCMOSCamera(var.shape[1], var.shape[0], 0.1, readnoise=np.sqrt(var),
                            offset=off, gain=gain)
        batch = G.ROIBatch(data, xc, yc, np.ones(len(xc), np.int32), cam)
        res = G.fit(fitter, batch)
    return res.params, res.uncertainties


@pytest.mark.parametrize("model", [0, 1, 2], ids=["xynb", "xynbs", "xynbsxsy"])
def test_model_validation_protocol_gpu(model):
    res = SC.check_model_validation(gpu_fit_api, model)
    assert all(v["pass"] for v in res.values()), res


def test_scmos_photometry_protocol_gpu():
    res = SC.check_scmos_photometry(gpu_fit_api)
    assert res["pass"], res


def test_scmos_variance_map_indexing_protocol_gpu():
    res = SC.check_variance_indexing(gpu_fit_api)
    assert res["pass"], res


def test_precision_improves_with_photons_gpu():
    res = SC.check_precision_vs_photons(gpu_fit_api)
    assert res["pass"], res


def test_astigmatic_validation_protocol_gpu():
    """test/model_validation_tests.jl:97-135 through fit(): bias and std/CRLB
    of x, y, z, N, bg with the reference's astigmatic calibration."""
    res = SC.check_astig_validation(gpu_fit_api)
    assert all(v["pass"] for v in res.values()), res


def test_result_columns_and_smld():
    psf, truth, data = SC.model_validation_data(1, n=200, box=11, seed=5)
    fitter = G.GaussMLEFitter(psf_model=G.GaussianXYNBS())
    res = G.fit(fitter, data)
    assert res.params.shape == (200, 5) and res.uncertainties.shape == (200, 5)
    assert np.all((res.pvalues >= 0) & (res.pvalues <= 1))
    smld = res.to_smld()
    assert smld.emitter_type == "Emitter2DFitSigma" and len(smld) == 200
    e = smld.emitters
    # positions in microns on the synthetic camera (x corners 1, 12, 23, ...)
    k = np.arange(200)
    np.testing.assert_allclose(e["x"], (k * 11 + res.params[:, 0] - 1) * np.float32(0.1),
                               rtol=1e-6)
    np.testing.assert_allclose(e["σ"], res.params[:, 4] * np.float32(0.1), rtol=1e-6)
    assert (res.flags & 1).all()

"""The compiled boundary without a GPU: the MEX gateways of mex/ (built
against the project's mx stub) and the standalone driver build, and they
reject bad inputs with MATLAB-style errors before any GPU work - a wrong
input count, a wrong class, a missing struct field, a bad option.  With
valid inputs on a machine without a GPU the library's status comes back as
an error too (BAMF_ERR_NO_DEVICE), so no call here reaches a kernel."""
import numpy as np
import pytest

from mex_harness import Gateway, MexError, run_driver


def _mcmc():
    from bamf_gb300 import rjstruct
    rj = rjstruct.c0_rjstruct()
    return {"PSFsigma": 1.3, "N_Trials": 10.0, "N_Burnin": 10.0, "I_stdFg": 10.0, "I_stdBg": 10.0,
            "X_stdFg": 0.1, "X_stdBg": 0.1, "P_Burnin": np.asarray(rj.P_Burnin, np.float32),
            "P_Trials": np.asarray(rj.P_Trials, np.float32), "Rho": 3 / 256, "Bnd_out": 2.0, "Grid_Zoom": 20.0,
            "Split_std": 0.5, "Icutoff": 0.0, "BG_std": 1.0, "ABBG_std": 0.0, "DX": 10.0, "DriftX": 0.0,
            "DriftY": 0.0, "PSFsize": np.array([10, 10, 2, 2], np.int32), "IsBackg": 0.0}


def _crjmcmc_args(**over):
    pdf = np.ones(100, np.float32) / 1000
    a = {"Data": np.full((16, 16), 10, np.float32),
         "E": {"N": 0.0, "I": np.zeros(0, np.float32), "X": np.zeros(0, np.float32),
               "Y": np.zeros(0, np.float32), "BG": 10.0},
         "MCMC": _mcmc(), "Xsize": 16.0, "Ysize": 16.0, "Off": pdf, "Sig": pdf, "Back": pdf,
         "sCMOS": np.zeros((16, 16), np.float32), "PSF": np.zeros((10, 10, 2, 2), np.float32), "Opt": 0.0}
    a.update(over)
    return [a[k] for k in ("Data", "E", "MCMC", "Xsize", "Ysize", "Off", "Sig", "Back", "sCMOS", "PSF", "Opt")]


@pytest.fixture(scope="module")
def crj():
    return Gateway("cRJMCMC_bamf")


def _expect(gw, ident, *args, nlhs=5):
    with pytest.raises(MexError) as e:
        gw(nlhs, *args)
    assert e.value.ident == ident, str(e.value)


def test_crjmcmc_gateway_rejects_bad_inputs(crj):
    _expect(crj, "bamf:cRJMCMC:nrhs", *_crjmcmc_args()[:10])
    _expect(crj, "bamf:cRJMCMC:type", *_crjmcmc_args(Data=np.full((16, 16), 10.0)))
    _expect(crj, "bamf:cRJMCMC:size", *_crjmcmc_args(Data=np.zeros((4, 4), np.float32)))
    m = _mcmc()
    del m["Split_std"]
    _expect(crj, "bamf:cRJMCMC:field", *_crjmcmc_args(MCMC=m))
    m = _mcmc()
    m["PSFsize"] = np.array([10, 10, 2, 2], np.float64)
    _expect(crj, "bamf:cRJMCMC:field", *_crjmcmc_args(MCMC=m))
    _expect(crj, "bamf:cRJMCMC:field", *_crjmcmc_args(E={"N": 0.0, "I": [], "X": [], "Y": []}))
    _expect(crj, "bamf:cRJMCMC:size", *_crjmcmc_args(E={"N": 2.0, "I": np.ones(1, np.float32),
                                                        "X": np.ones(2, np.float32),
                                                        "Y": np.ones(2, np.float32), "BG": 1.0}))
    _expect(crj, "bamf:cRJMCMC:OptModel", *_crjmcmc_args(Opt=3.0))
    _expect(crj, "bamf:cRJMCMC:Arith", *_crjmcmc_args(), "wrong")
    _expect(crj, "bamf:cRJMCMC:nlhs", *_crjmcmc_args(), nlhs=6)


def test_crjmcmc_gateway_reports_library_status_without_a_gpu(crj):
    from bamf_gb300 import abi
    if abi.lib().bamf_device_count() > 0:
        pytest.skip("a GPU is visible: the call would run")
    _expect(crj, "bamf:cRJMCMC:status", *_crjmcmc_args())


def test_findroi_and_gaussmle_gateways_reject_bad_inputs():
    fr = Gateway("findROI_bamf")
    _expect(fr, "bamf:findROI:nrhs", nlhs=3)
    _expect(fr, "bamf:findROI:type", np.zeros((32, 32, 2)), nlhs=3)
    _expect(fr, "bamf:findROI:size", np.zeros((8, 8, 2), np.float32), 1.3, 2.6, 9.0, nlhs=3)
    _expect(fr, "bamf:findROI:type", np.zeros((32, 32, 2), np.float32), "x", nlhs=3)
    g = Gateway("gaussMLE_bamf")
    d = np.zeros((7, 7, 4), np.float32)
    _expect(g, "bamf:gaussMLE:nrhs", d, "Basic", "CCD", nlhs=2)
    _expect(g, "bamf:gaussMLE:FitType", d, "Foo", "CCD", 1.3, nlhs=2)
    _expect(g, "bamf:gaussMLE:CameraType", d, "Basic", "EMCCD", 1.3, nlhs=2)
    _expect(g, "bamf:gaussMLE:size", np.zeros((7, 6, 4), np.float32), "Basic", "CCD", 1.3, nlhs=2)
    _expect(g, "bamf:gaussMLE:type", d.astype(np.float64), "Basic", "CCD", 1.3, nlhs=2)
    _expect(g, "bamf:gaussMLE:nrhs", d, "Z", "CCD", 1.3, nlhs=2)
    _expect(g, "bamf:gaussMLE:field", d, "Z", "CCD", np.array([1.3, 1.3]), {"Ax": 1.0}, nlhs=2)
    _expect(g, "bamf:gaussMLE:size", d, "Basic", "SCMOS", 1.3, np.zeros((8, 9), np.float32),
            np.zeros((4, 2), np.float32), nlhs=2)
    _expect(g, "bamf:gaussMLE:option", d, "Basic", "CCD", 1.3, "Iter", 5.0, nlhs=2)


def test_driver_builds_and_rejects_bad_input(tmp_path):
    r = run_driver(check=False)
    assert r.returncode == 2 and "usage" in r.stderr
    bad = tmp_path / "in.bin"
    bad.write_bytes(b"not an input")
    r = run_driver("rjmcmc", bad, tmp_path / "out.bin", check=False)
    assert r.returncode == 1 and "not a bamf_driver rjmcmc input" in r.stderr

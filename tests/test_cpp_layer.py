"""The C++ drop-in layer (ILeapCalibrator / LeapCalibratorFactory /
ComputeImplementation) through its driver, on the CPU: argument handling,
the new "gb300" value, and the reference's errors for implementations this
library does not build."""
import json
import os
import subprocess

import numpy as np
import pytest

import leap_gb300 as lg
from leap_gb300 import synth

DRIVER = os.path.join(os.path.dirname(lg.LIB_PATH), "leap_calibrate_driver")


def run(args, **kw):
    return subprocess.run([DRIVER] + args, capture_output=True, text=True, timeout=120, **kw)


def _gpu():
    import torch
    return torch.cuda.is_available()


@pytest.fixture(scope="module")
def leapms(tmp_path_factory):
    obs, dirs = synth.small_case(stations=8, timesteps=3, channels=6, directions=2, vis_dtype=np.complex64)
    p = str(tmp_path_factory.mktemp("ms") / "small.leapms")
    synth.write_leapms(obs, p)
    return p, obs, dirs


def test_driver_built():
    assert os.path.exists(DRIVER)


@pytest.mark.parametrize("impl,msg", [("cpu", "cpu implementation not built"), ("casa", "cpu implementation not built"),
                                      ("cuda", "cuda build option not enabled"), ("bogus", "unknown compute implementation")])
def test_factory_errors_match_reference(leapms, impl, msg):
    path, obs, dirs = leapms
    r = run(["-f", path, "-i", impl, "-d", json.dumps(dirs.tolist())])
    assert r.returncode != 0
    assert msg in r.stderr


def test_gb300_without_gpu_reports_device_error(leapms):
    if _gpu():
        pytest.skip("a GPU is present")
    path, obs, dirs = leapms
    r = run(["-f", path, "-i", "gb300", "-d", json.dumps(dirs.tolist())])
    assert r.returncode != 0 and "no CUDA device" in r.stderr


def test_cli_overrides_config(leapms, tmp_path):
    """defaults < config < command line: the config asks for cpu, the command line for gb300."""
    path, obs, dirs = leapms
    cfg = tmp_path / "cfg.json"
    cfg.write_text(json.dumps({"filePath": path, "computeImplementation": "cpu", "directions": dirs.tolist()}))
    r = run(["--config", str(cfg)])
    assert r.returncode != 0 and "cpu implementation not built" in r.stderr
    r = run(["--config", str(cfg), "-i", "gb300"])
    assert "cpu implementation not built" not in r.stderr


def test_missing_file_is_a_file_error(tmp_path):
    r = run(["-f", str(tmp_path / "nope.leapms"), "-i", "gb300", "-d", "[[0.0, 0.0]]"])
    assert r.returncode != 0 and "cannot open" in r.stderr


def test_measurement_set_validation(tmp_path):
    """Rows must be a whole number of timesteps (MeasurementSet.cc:95-102)."""
    obs, dirs = synth.small_case(stations=6, timesteps=2, channels=3, directions=1)
    obs.timesteps = 2
    p = tmp_path / "bad.leapms"
    synth.write_leapms(obs, str(p))
    raw = bytearray(p.read_bytes())
    # rows field (third uint32 of the header) claims one row fewer than written
    rows = int.from_bytes(raw[16:20], "little")
    raw[16:20] = (rows - 1).to_bytes(4, "little")
    p.write_bytes(bytes(raw))
    r = run(["-f", str(p), "-i", "gb300", "-d", json.dumps(dirs.tolist())])
    assert r.returncode != 0


def test_bad_slice_rejected(leapms):
    path, obs, dirs = leapms
    r = run(["-f", path, "-i", "gb300", "-d", json.dumps(dirs.tolist()), "-s", "0"])
    assert r.returncode != 0 and "non zero" in r.stderr

"""The C++ drop-in: LeapCalibratorFactory::Create(gb300)->Calibrate(...) on a
MeasurementSet stand-in, compared with the oracle's CpuLeapCalibrator
restatement (FP64 form within 1e-10 rad, mixed within 1e-5 rad)."""
import json
import os
import subprocess

import numpy as np
import pytest

import oracle
import leap_gb300 as lg
from leap_gb300 import synth

pytestmark = pytest.mark.gpu
DRIVER = os.path.join(os.path.dirname(lg.LIB_PATH), "leap_calibrate_driver")


def calibrate(path, dirs, interval="-1", precision="fp64", extra=()):
    r = subprocess.run([DRIVER, "-f", path, "-i", "gb300", "-d", json.dumps(np.asarray(dirs).tolist()),
                        "-s", interval, "-p", precision, *extra], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout)


def compare(got, exp, tol):
    assert len(got) == len(exp) > 0
    for g, e in zip(got, exp):
        assert g["epoch"]["start"] == e["epoch"]["start"] and g["epoch"]["end"] == e["epoch"]["end"]
        for gb, eb in zip(g["calibration"], e["calibration"]):
            assert gb["direction"] == eb["direction"]
            assert np.abs(np.array(gb["beamCalibration"]) - np.array(eb["beamCalibration"])).max() <= tol


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
@pytest.mark.parametrize("interval,triple", [("-1", (0, -1, -1)), ("1", (0, 1, -1)), ("[0, 2]", (0, 2, 2))])
def test_drop_in_fp64_matches_oracle(tmp_path, dtype, interval, triple):
    obs, dirs = synth.small_case(stations=14, timesteps=4, channels=9, directions=3, vis_dtype=dtype, seed_shift=7)
    path = str(tmp_path / "obs.leapms")
    synth.write_leapms(obs, path)
    compare(calibrate(path, dirs, interval), oracle.calibrate(obs, dirs, triple), 1e-10)


def test_drop_in_askap_small_and_reference_antenna(tmp_path):
    obs, dirs = synth.askap_small()
    path = str(tmp_path / "askap.leapms")
    synth.write_leapms(obs, path)
    compare(calibrate(path, dirs), oracle.calibrate(obs, dirs), 1e-10)
    compare(calibrate(path, dirs, extra=("-a", "3")), oracle.calibrate(obs, dirs, reference_antenna=3), 1e-10)


def test_drop_in_mixed_via_config(tmp_path):
    obs, dirs = synth.small_case(stations=30, timesteps=3, channels=40, directions=6, vis_dtype=np.complex64)
    path = str(tmp_path / "obs.leapms")
    synth.write_leapms(obs, path)
    cfg = tmp_path / "config.json"
    cfg.write_text(json.dumps({"filePath": path, "computeImplementation": "gb300", "directions": dirs.tolist(),
                               "precision": "mixed"}))
    r = subprocess.run([DRIVER, "--config", str(cfg)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    compare(json.loads(r.stdout), oracle.calibrate(obs, dirs), 1e-5)


def test_drop_in_file_cache(tmp_path):
    """isFileSystemCacheEnabled: the second run reads the pseudoinverse from A.hash/Ad.cache."""
    obs, dirs = synth.small_case(stations=10, timesteps=2, channels=5, directions=2)
    path = str(tmp_path / "obs.leapms")
    synth.write_leapms(obs, path)
    exp = oracle.calibrate(obs, dirs)
    for _ in range(2):
        r = subprocess.run([DRIVER, "-f", path, "-i", "gb300", "-d", json.dumps(dirs.tolist()), "--cache"],
                           capture_output=True, text=True, timeout=600, cwd=str(tmp_path))
        assert r.returncode == 0, r.stderr
        compare(json.loads(r.stdout), exp, 1e-10)
    assert (tmp_path / "A.hash").exists() and (tmp_path / "Ad.cache").exists()

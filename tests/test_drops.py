"""leap_drops counterparts: config splitting and gathering (CPU), the .leapms
reader, and (GPU) the in-process calibration drop against the oracle."""
import json

import numpy as np
import pytest

import oracle
from leap_gb300 import drops, synth


def test_directions_csv_and_config_split_follow_produce_config():
    text = "0.1,0.2\nbad\n0.3,0.4,0.5\n0.5,0.6\n0.7,0.8\n"
    d = drops.read_directions_csv(text)
    assert d == [[0.1, 0.2], [0.5, 0.6], [0.7, 0.8]]
    cfgs = [json.loads(c) for c in drops.produce_configs(d, 2, 36)]
    assert [c["directions"] for c in cfgs] == [[[0.1, 0.2]], [[0.5, 0.6], [0.7, 0.8]]]
    assert all(c["numStations"] == 36 and c["implementation"] == "gb300" and c["autoCorrelation"] for c in cfgs)
    assert json.loads(drops.gather(['[1]', '[2, 3]'])) == [[1], [2, 3]]


def test_leapms_round_trip(tmp_path):
    obs, _ = synth.small_case(stations=7, timesteps=3, channels=5, directions=1, vis_dtype=np.complex64)
    path = str(tmp_path / "x.leapms")
    synth.write_leapms(obs, path)
    back = synth.read_leapms(path)
    assert back.nbaselines == obs.nbaselines and back.timesteps == obs.timesteps
    np.testing.assert_array_equal(back.ms_vis, obs.vis.transpose(1, 0, 2))
    np.testing.assert_array_equal(back.uvw, obs.uvw)
    np.testing.assert_array_equal(back.epochs, obs.epochs)
    np.testing.assert_array_equal(back.flags, obs.flags)


def test_unserved_implementation_is_rejected_without_a_gpu():
    with pytest.raises(ValueError):
        app = drops.CallLeapInProcess.__new__(drops.CallLeapInProcess)
        app.obs = None
        app.run(json.dumps({"implementation": "cpu", "directions": [[0.0, 0.0]]}))


@pytest.mark.gpu
def test_call_leap_in_process_matches_oracle(tmp_path):
    obs, dirs = synth.small_case(stations=14, timesteps=4, channels=9, directions=5, vis_dtype=np.complex64)
    path = str(tmp_path / "obs.leapms")
    synth.write_leapms(obs, path)
    configs = drops.produce_configs(dirs.tolist(), 2, obs.num_stations)
    app = drops.CallLeapInProcess(path, solution_interval=(0, 2, -1))
    try:
        out = json.loads(drops.gather([app.run(c) for c in configs]))
    finally:
        app.close()
    exp = oracle.calibrate(obs, dirs, (0, 2, -1))
    got = [cal for part in out for cal in part]  # two instances x two solution intervals
    assert len(got) == 4
    for inst in range(2):
        for s in range(2):
            g = out[inst][s]
            e = exp[s]
            assert g["epoch"] == e["epoch"]
            for gb in g["calibration"]:
                eb = next(b for b in e["calibration"] if b["direction"] == gb["direction"])
                assert np.abs(np.array(gb["beamCalibration"]) - np.array(eb["beamCalibration"])).max() <= 1e-10

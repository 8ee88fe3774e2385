"""In-process counterparts of the reference's DALiuGE drops (R/leap_drops/).

The reference splits a direction list into per-instance configs (ProduceConfig.py:60-123), runs one
LeapAccelerateCLI subprocess per config (CallLeap.py:37-90) and gathers the JSON outputs (LeapGather.py:30-54).
Here the middle step calls the GB300 path in-process through the C ABI (leap_gb300.GpuLeapCalibrator), with no
subprocess and no re-reading of the MeasurementSet per instance; the config and result formats are the
reference's, so the producer and gatherer are interchangeable with the reference's drops.

DALiuGE itself is optional: the functions below take and return plain strings; when ``dlg`` is importable,
``CallLeapGB300`` wraps them as a BarrierAppDROP.
"""
from __future__ import annotations

import csv
import json
import math
from typing import List, Optional, Sequence

from . import _abi
from .calibrator import GpuLeapCalibrator

__all__ = ["read_directions_csv", "produce_configs", "CallLeapInProcess", "gather"]

# Values of the config's "implementation" key this library serves (compute_implementation.cc aliases
# "casa"/"eigen" name the reference's CPU path, which is not built here).
SERVED_IMPLEMENTATIONS = ("gb300",)


def read_directions_csv(text: str) -> List[List[float]]:
    """Rows of two numbers (ra, dec); other rows are skipped (ProduceConfig._readDirections)."""
    out = []
    for row in csv.reader(text.split("\n")):
        if len(row) != 2:
            continue
        out.append([float(row[0]), float(row[1])])
    return out


def produce_configs(directions: Sequence[Sequence[float]], instances: int, num_stations: int,
                    implementation: str = "gb300", auto_correlation: bool = True) -> List[str]:
    """Split the directions over `instances` configs the way ProduceConfig.run does:
    instance i takes [floor(i * n / k), floor((i + 1) * n / k))."""
    per = float(len(directions)) / float(instances)
    out, start = [], 0
    for i in range(instances):
        end = int(math.floor((i + 1) * per))
        out.append(json.dumps({"numStations": num_stations, "directions": [list(d) for d in directions[start:end]],
                               "implementation": implementation, "autoCorrelation": auto_correlation}))
        start = end
    return out


class CallLeapInProcess:
    """Calibrate one config against a MeasurementSet, in-process (CallLeap.run without the subprocess).

    `measurement_set` is a ".leapms" path or an Observation (leap_gb300.synth); the result is the
    CalibrationCollection JSON that LeapAccelerateCLI writes."""

    def __init__(self, measurement_set, device: int = 0, precision: int = _abi.LEAP_PRECISION_FP64,
                 solution_interval=(0, -1, -1), reference_antenna: Optional[int] = None,
                 minimum_baseline_threshold: float = 0.0):
        from . import synth
        self.obs = synth.read_leapms(measurement_set) if isinstance(measurement_set, str) else measurement_set
        self.solution_interval = solution_interval
        self.reference_antenna = reference_antenna
        self.minimum_baseline_threshold = minimum_baseline_threshold
        self.calibrator = GpuLeapCalibrator(device, precision)

    def run(self, config_json: str) -> str:
        config = json.loads(config_json)
        impl = config.get("implementation", config.get("computeImplementation", "gb300"))
        if impl not in SERVED_IMPLEMENTATIONS:
            raise ValueError(f"implementation {impl!r} is not built in this library (use 'gb300')")
        ns = config.get("numStations")
        if ns is not None and int(ns) != self.obs.num_stations:
            raise ValueError(f"config numStations {ns} != measurement set stations {self.obs.num_stations}")
        if not config.get("autoCorrelation", True):
            raise ValueError("autoCorrelation false is not supported by the .leapms stand-in")
        directions = config["directions"]
        if not directions:
            return json.dumps([])
        result = self.calibrator.calibrate(self.obs, directions, self.solution_interval,
                                           self.minimum_baseline_threshold, self.reference_antenna)
        return json.dumps(result)

    def close(self):
        self.calibrator.ctx.close()


def gather(outputs: Sequence[str]) -> str:
    """LeapGather.run: the list of every instance's parsed output, in input order."""
    return json.dumps([json.loads(o) for o in outputs])


try:  # pragma: no cover - DALiuGE is not installed in the test environments
    from dlg.drop import BarrierAppDROP
    from dlg.droputils import DROPFile

    class CallLeapGB300(BarrierAppDROP):
        """BarrierAppDROP: one config in, the CalibrationCollection JSON out (in-process GB300 path)."""
        measurementSetFilename = ""

        def run(self):
            if len(self.inputs) != 1 or len(self.outputs) != 1:
                raise Exception("One input and one output are expected by this application")
            with DROPFile(self.inputs[0]) as f:
                config = f.read()
            app = CallLeapInProcess(self.measurementSetFilename)
            try:
                self.outputs[0].write(app.run(config).encode())
            finally:
                app.close()
except ImportError:
    pass

"""ORACLE — TEST INFRASTRUCTURE ONLY.

The reference's kernelTuner bookkeeping (src/utilities/kernelTuner.cpp:4-126) restated in plain
Python, with the time of each timed call supplied by the caller instead of CUDA events, so that
the product's tuner can be checked against it on the CPU with the same sequences of times.
"""
from __future__ import annotations

STARTUP, IDLE, SCANNING = 0, 1, 2


class KernelTunerOracle:
    def __init__(self, start: int, end: int, step: int, n_samples: int, period: int):
        # constructor (kernelTuner.cpp:4-24): the sample count is rounded UP to even when odd
        self.state = STARTUP
        self.current_sample = 0
        self.current_index = 0
        self.calls_since = 0
        self.period = period
        self.parameter = start
        self.candidates = list(range(start, end + 1, step))
        self.samples_per_value = n_samples + 1 if n_samples % 2 == 1 else n_samples
        self.samples = [[0.0] * self.samples_per_value for _ in self.candidates]
        self.medians = [0.0] * len(self.candidates)

    def timing(self) -> bool:
        # begin() records the start event unless IDLE (kernelTuner.cpp:32-36)
        return self.state != IDLE

    def _optimum(self) -> int:
        # computeOptimalParameter (kernelTuner.cpp:100-126): median = element size/2 after
        # nth_element, strict < keeps the earlier candidate on ties
        for i, t in enumerate(self.samples):
            self.medians[i] = sorted(t)[len(t) // 2]
        best = 0
        for i in range(1, len(self.candidates)):
            if self.medians[i] < self.medians[best]:
                best = i
        return self.candidates[best]

    def call(self, ms: float):
        # end() (kernelTuner.cpp:38-98)
        if self.state != IDLE:
            self.samples[self.current_index][self.current_sample] = ms
        if self.state == STARTUP:
            self.current_sample += 1
            if self.current_sample >= self.samples_per_value:
                self.current_sample = 0
                self.current_index += 1
                if self.current_index >= len(self.candidates):
                    self.current_index = 0
                    self.state = IDLE
                    self.parameter = self._optimum()
                else:
                    self.parameter = self.candidates[self.current_index]
        elif self.state == SCANNING:
            self.current_index += 1
            if self.current_index >= len(self.candidates):
                self.current_index = 0
                self.state = IDLE
                self.parameter = self._optimum()
                self.current_sample = (self.current_sample + 1) % self.samples_per_value
            else:
                self.parameter = self.candidates[self.current_index]
        else:
            self.calls_since += 1
            if self.calls_since > self.period:
                self.calls_since = 0
                self.parameter = self.candidates[self.current_index]
                self.state = SCANNING

// Launch-parameter autotuner: the state machine of the reference's kernelTuner
// (src/utilities/kernelTuner.{h,cpp}), with the timing source separated from the bookkeeping so
// that the bookkeeping runs (and is tested) without a GPU.
//
// Behaviour kept from the reference (kernelTuner.cpp:4-126):
//   * candidates start, start+step, ..., <= end; the first candidate is used first;
//   * samplesPerValue = nSamples, plus one when nSamples is odd (the reference's comment says it
//     forces an odd count; its code rounds odd counts up to even, and that is what is kept);
//   * STARTUP: each candidate is timed samplesPerValue times in turn, then the candidate with the
//     lowest median (element size/2 after nth_element; ties keep the earlier candidate) is used and
//     the tuner goes IDLE;
//   * IDLE: after more than `period` further calls it goes SCANNING from the candidate index it
//     left off at: one new sample per candidate (overwriting sample slot currentSample), then the
//     optimum is recomputed, currentSample advances modulo samplesPerValue, and it is IDLE again.
#pragma once
#include <vector>

namespace svm {

class KernelTuner {
public:
    KernelTuner(int start, int end, int step, int nSamples, int period);
    int parameter() const { return parameterValue_; }
    bool samplingComplete() const { return state_ != STARTUP; }
    bool timing() const { return state_ != IDLE; }  // whether the next call is timed
    // One call of the tuned kernel: `ms` is its measured time when timing() was true (ignored
    // otherwise).  The reference's end() after begin().
    void call(float ms);
    const std::vector<int>& candidates() const { return candidates_; }
    const std::vector<float>& medians() const { return medians_; }
    int samplesPerValue() const { return samplesPerValue_; }

private:
    enum State { STARTUP, IDLE, SCANNING };
    int optimum();
    int parameterValue_;
    int samplesPerValue_;
    int period_;
    std::vector<int> candidates_;
    State state_ = STARTUP;
    int currentSample_ = 0;
    int currentIndex_ = 0;
    int callsSinceLastSample_ = 0;
    std::vector<std::vector<float>> samples_;
    std::vector<float> medians_;
};

}  // namespace svm

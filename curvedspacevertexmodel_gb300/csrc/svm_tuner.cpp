// KernelTuner bookkeeping and its C ABI (svm_tuner_* in include/svm.h).  The timed variant of a
// call records CUDA events on the tuner's stream around the caller's launch.
#include "svm_tuner.h"

#include <algorithm>
#include <cuda_runtime.h>

#include "../../include/svm.h"

namespace svm {

KernelTuner::KernelTuner(int start, int end, int step, int nSamples, int period)
    : parameterValue_(start), samplesPerValue_(nSamples), period_(period) {
    for (int v = start; v <= end; v += step) candidates_.push_back(v);
    if (samplesPerValue_ % 2 == 1) samplesPerValue_ += 1;
    samples_.assign(candidates_.size(), std::vector<float>(samplesPerValue_, 0.f));
    medians_.assign(candidates_.size(), 0.f);
}

int KernelTuner::optimum() {
    for (size_t i = 0; i < candidates_.size(); ++i) {
        std::vector<float> t = samples_[i];
        const size_t mid = t.size() / 2;
        std::nth_element(t.begin(), t.begin() + mid, t.end());
        medians_[i] = t[mid];
    }
    size_t best = 0;
    for (size_t i = 1; i < candidates_.size(); ++i)
        if (medians_[i] < medians_[best]) best = i;
    return candidates_[best];
}

void KernelTuner::call(float ms) {
    if (state_ != IDLE) samples_[currentIndex_][currentSample_] = ms;
    if (state_ == STARTUP) {
        if (++currentSample_ >= samplesPerValue_) {
            currentSample_ = 0;
            if (++currentIndex_ >= (int)candidates_.size()) {
                currentIndex_ = 0;
                state_ = IDLE;
                parameterValue_ = optimum();
            } else {
                parameterValue_ = candidates_[currentIndex_];
            }
        }
    } else if (state_ == SCANNING) {
        if (++currentIndex_ >= (int)candidates_.size()) {
            currentIndex_ = 0;
            state_ = IDLE;
            parameterValue_ = optimum();
            currentSample_ = (currentSample_ + 1) % samplesPerValue_;
        } else {
            parameterValue_ = candidates_[currentIndex_];
        }
    } else {
        if (++callsSinceLastSample_ > period_) {
            callsSinceLastSample_ = 0;
            parameterValue_ = candidates_[currentIndex_];
            state_ = SCANNING;
        }
    }
}

}  // namespace svm

struct svm_tuner {
    svm::KernelTuner t;
    cudaStream_t stream = nullptr;
    cudaEvent_t start = nullptr, stop = nullptr;
    bool begun = false;
    svm_tuner(int a, int b, int c, int d, int e) : t(a, b, c, d, e) {}
};

extern "C" {

int svm_tuner_create(int start, int end, int step, int nSamples, int period, void* stream, svm_tuner** out) {
    if (!out || step <= 0 || end < start || nSamples < 1 || period < 0) return SVM_ERR_ARG;
    svm_tuner* t = new svm_tuner(start, end, step, nSamples, period);
    t->stream = static_cast<cudaStream_t>(stream);
    *out = t;
    return SVM_OK;
}

int svm_tuner_destroy(svm_tuner* t) {
    if (!t) return SVM_ERR_ARG;
    if (t->start) cudaEventDestroy(t->start);
    if (t->stop) cudaEventDestroy(t->stop);
    delete t;
    return SVM_OK;
}

int svm_tuner_begin(svm_tuner* t) {
    if (!t) return SVM_ERR_ARG;
    t->begun = t->t.timing();
    if (!t->begun) return SVM_OK;
    if (!t->start && (cudaEventCreate(&t->start) != cudaSuccess || cudaEventCreate(&t->stop) != cudaSuccess))
        return SVM_ERR_CUDA;
    return cudaEventRecord(t->start, t->stream) == cudaSuccess ? SVM_OK : SVM_ERR_CUDA;
}

int svm_tuner_end(svm_tuner* t) {
    if (!t) return SVM_ERR_ARG;
    float ms = 0.f;
    if (t->begun) {
        if (cudaEventRecord(t->stop, t->stream) != cudaSuccess || cudaEventSynchronize(t->stop) != cudaSuccess ||
            cudaEventElapsedTime(&ms, t->start, t->stop) != cudaSuccess)
            return SVM_ERR_CUDA;
    }
    t->begun = false;
    t->t.call(ms);
    return SVM_OK;
}

int svm_tuner_record(svm_tuner* t, float ms) {
    if (!t) return SVM_ERR_ARG;
    t->t.call(ms);
    return SVM_OK;
}

int svm_tuner_parameter(svm_tuner* t, int* value) {
    if (!t || !value) return SVM_ERR_ARG;
    *value = t->t.parameter();
    return SVM_OK;
}

int svm_tuner_sampling_complete(svm_tuner* t, int* done) {
    if (!t || !done) return SVM_ERR_ARG;
    *done = t->t.samplingComplete() ? 1 : 0;
    return SVM_OK;
}

int svm_tuner_timing_data(svm_tuner* t, int* candidates, float* medians, int capacity, int* count) {
    if (!t || !count) return SVM_ERR_ARG;
    const int n = (int)t->t.candidates().size();
    *count = n;
    for (int i = 0; i < n && i < capacity; ++i) {
        if (candidates) candidates[i] = t->t.candidates()[i];
        if (medians) medians[i] = t->t.medians()[i];
    }
    return SVM_OK;
}

}  // extern "C"

// timer.h -- accumulating wall-clock timer with the interface of the reference's lib/timer.h.
#ifndef CSP_DROPIN_TIMER_H
#define CSP_DROPIN_TIMER_H

#include <chrono>

class Timer {
public:
    void start() {
        running_ = true;
        t0_ = clock::now();
    }
    // adds the time since start() to the accumulated total
    void stop() {
        if (!running_) return;
        running_ = false;
        total_ += clock::now() - t0_;
    }
    void reset() { total_ = std::chrono::duration<double>(0); }
    // while running: time since start(); otherwise the accumulated total
    unsigned long long get_time_milli_sec() const {
        const auto d = running_ ? std::chrono::duration<double>(clock::now() - t0_) : total_;
        return (unsigned long long)std::chrono::duration_cast<std::chrono::milliseconds>(d).count();
    }
    double get_time_sec() const {
        return running_ ? std::chrono::duration<double>(clock::now() - t0_).count() : total_.count();
    }
    double operator()() const { return get_time_sec(); }

private:
    using clock = std::chrono::high_resolution_clock;
    bool running_ = false;
    clock::time_point t0_{};
    std::chrono::duration<double> total_{0};
};

#endif

// Small persistent thread pool for the CPU set-up code (grid rasterising, Laplace solve,
// efield).  parallel_for hands out [0, n) in fixed chunks; work items never depend on
// which thread runs them, so results are independent of the thread count.
#pragma once
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace mq {

class Pool {
public:
    explicit Pool(int threads) {
        int hw = (int)std::thread::hardware_concurrency();
        nthreads_ = threads > 0 ? threads : std::max(1, hw);
        for (int t = 1; t < nthreads_; ++t) workers_.emplace_back([this] { loop(); });
    }
    ~Pool() {
        {
            std::lock_guard<std::mutex> lk(m_);
            stop_ = true;
            ++gen_;
        }
        cv_.notify_all();
        for (auto& w : workers_) w.join();
    }
    int size() const { return nthreads_; }

    // Run f(i) for i in [0, n).  Items are claimed one at a time through an atomic counter.
    void parallel_for(long n, const std::function<void(long)>& f) {
        if (n <= 0) return;
        if (nthreads_ == 1 || n == 1) {
            for (long i = 0; i < n; ++i) f(i);
            return;
        }
        {
            std::lock_guard<std::mutex> lk(m_);
            job_ = &f;
            n_ = n;
            next_.store(0);
            active_ = nthreads_ - 1;
            ++gen_;
        }
        cv_.notify_all();
        work();
        std::unique_lock<std::mutex> lk(m_);
        done_cv_.wait(lk, [this] { return active_ == 0; });
        job_ = nullptr;
    }

private:
    void work() {
        const std::function<void(long)>* f = job_;
        for (;;) {
            long i = next_.fetch_add(1);
            if (i >= n_) break;
            (*f)(i);
        }
    }
    void loop() {
        unsigned long seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(m_);
                cv_.wait(lk, [&] { return gen_ != seen; });
                seen = gen_;
                if (stop_) return;
            }
            work();
            {
                std::lock_guard<std::mutex> lk(m_);
                if (--active_ == 0) done_cv_.notify_all();
            }
        }
    }
    int nthreads_ = 1;
    std::vector<std::thread> workers_;
    std::mutex m_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(long)>* job_ = nullptr;
    long n_ = 0;
    std::atomic<long> next_{0};
    int active_ = 0;
    unsigned long gen_ = 0;
    bool stop_ = false;
};

}  // namespace mq

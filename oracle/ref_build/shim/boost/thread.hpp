// Stand-in for the parts of Boost.Thread the reference's scatter devices use, built on
// the C++ standard library: mutex with scoped_lock, condition_variable, barrier, thread
// with interrupt(), this_thread, posix_time::milliseconds and shared_ptr.
//
// Interruption follows Boost's contract as far as the devices rely on it: interrupt()
// marks the thread, and its next wait on a condition variable or a barrier throws
// boost::thread_interrupted, which ends the thread function. The devices' stop_workers()
// interrupts every worker and then deletes it; deleting an interrupted thread joins it
// here, so the harness can unload the library with no thread left running.
#pragma once
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <functional>
#include <memory>
#include <mutex>
#include <thread>

#include <boost/bind.hpp>  // Boost.Thread brings boost::bind with it

namespace boost {

struct thread_interrupted {};

using std::shared_ptr;

namespace shim_detail {
struct InterruptFlag {
    std::atomic<bool> requested{false};
};
inline std::shared_ptr<InterruptFlag>& current_flag() {
    thread_local std::shared_ptr<InterruptFlag> f = std::make_shared<InterruptFlag>();
    return f;
}
inline void interruption_point() {
    if (current_flag()->requested.load()) throw thread_interrupted();
}
constexpr std::chrono::milliseconds kPoll(2);
}  // namespace shim_detail

class mutex {
    std::mutex m_;

public:
    void lock() { m_.lock(); }
    void unlock() { m_.unlock(); }
    bool try_lock() { return m_.try_lock(); }
    typedef std::unique_lock<mutex> scoped_lock;
};

class condition_variable {
    std::condition_variable_any cv_;

public:
    void notify_all() { cv_.notify_all(); }
    void notify_one() { cv_.notify_one(); }
    // May return spuriously (as Boost's may); callers re-check their predicate.
    template <class Lock>
    void wait(Lock& lock) {
        shim_detail::interruption_point();
        cv_.wait_for(lock, shim_detail::kPoll);
        shim_detail::interruption_point();
    }
};

class barrier {
    std::mutex m_;
    std::condition_variable cv_;
    unsigned n_, left_, generation_ = 0;

public:
    explicit barrier(unsigned n) : n_(n), left_(n) {}
    bool wait() {
        std::unique_lock<std::mutex> lk(m_);
        const unsigned g = generation_;
        if (--left_ == 0) {
            ++generation_;
            left_ = n_;
            cv_.notify_all();
            return true;
        }
        while (g == generation_) {
            cv_.wait_for(lk, shim_detail::kPoll);
            if (g == generation_ && shim_detail::current_flag()->requested.load()) throw thread_interrupted();
        }
        return false;
    }
};

class thread {
    std::shared_ptr<shim_detail::InterruptFlag> flag_;
    std::thread t_;

public:
    typedef std::thread::id id;
    template <class F>
    explicit thread(F f) : flag_(std::make_shared<shim_detail::InterruptFlag>()) {
        std::shared_ptr<shim_detail::InterruptFlag> flag = flag_;
        t_ = std::thread([flag, f]() mutable {
            shim_detail::current_flag() = flag;
            try {
                f();
            } catch (thread_interrupted&) {
            }
        });
    }
    id get_id() const { return t_.get_id(); }
    void interrupt() { flag_->requested = true; }
    void join() {
        if (t_.joinable()) t_.join();
    }
    ~thread() {
        if (!t_.joinable()) return;
        if (flag_->requested)
            t_.join();
        else
            t_.detach();
    }
};

namespace posix_time {
struct milliseconds {
    long ms;
    explicit milliseconds(long v) : ms(v) {}
};
}  // namespace posix_time

namespace this_thread {
inline std::thread::id get_id() { return std::this_thread::get_id(); }
inline void sleep(const posix_time::milliseconds& d) {
    std::this_thread::sleep_for(std::chrono::milliseconds(d.ms));
    shim_detail::interruption_point();
}
}  // namespace this_thread

}  // namespace boost

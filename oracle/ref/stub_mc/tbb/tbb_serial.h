// A serial stand-in for the parts of oneTBB that the MeshLib units compiled by
// oracle/ref/build_cpu_ref.py (the mesher, and the winding-number path with its mesh, tree and
// projection) use, so that the reference's CPU code can be compiled from its own sources for the
// oracle's golden vectors without the un-vendored TBB.  Every parallel algorithm runs its body once
// over the whole range on the calling thread.  The outputs do not depend on the thread count: the
// mesher's vertex ids are block-local counts shifted by prefix sums (its block partition is passed
// explicitly), and every winding-number / distance query is evaluated independently.
// TEST INFRASTRUCTURE ONLY.
#pragma once
#include <algorithm>
#include <cstddef>
#include <functional>
#include <iterator>
#include <list>
#include <thread>
#include <utility>

namespace tbb {

struct split {};

template <typename Value>
class blocked_range {
public:
    using const_iterator = Value;
    using size_type = std::size_t;
    blocked_range() = default;
    blocked_range(Value b, Value e, size_type grain = 1) : begin_(b), end_(e), grain_(grain) {}
    blocked_range(blocked_range& r, split) : begin_(r.begin_), end_(r.end_), grain_(r.grain_) {}
    Value begin() const { return begin_; }
    Value end() const { return end_; }
    size_type size() const { return size_type(end_ - begin_); }
    size_type grainsize() const { return grain_; }
    bool empty() const { return !(begin_ < end_); }
    bool is_divisible() const { return false; }

private:
    Value begin_{}, end_{};
    size_type grain_ = 1;
};

template <typename RowValue, typename ColValue = RowValue>
class blocked_range2d {
public:
    blocked_range2d(RowValue rb, RowValue re, ColValue cb, ColValue ce) : rows_(rb, re), cols_(cb, ce) {}
    const blocked_range<RowValue>& rows() const { return rows_; }
    const blocked_range<ColValue>& cols() const { return cols_; }

private:
    blocked_range<RowValue> rows_;
    blocked_range<ColValue> cols_;
};

class task_group_context {
public:
    task_group_context() = default;
    bool cancel_group_execution() { cancelled_ = true; return true; }
    bool is_group_execution_cancelled() const { return cancelled_; }
    void reset() { cancelled_ = false; }

private:
    bool cancelled_ = false;
};

struct auto_partitioner {};
struct simple_partitioner {};
struct static_partitioner {};
class affinity_partitioner {};

template <typename Range, typename Body>
void parallel_for(const Range& r, const Body& body) { body(r); }
template <typename Range, typename Body, typename P>
void parallel_for(const Range& r, const Body& body, P&&) { body(r); }
template <typename Range, typename Body, typename P>
void parallel_for(const Range& r, const Body& body, P&&, task_group_context&) { body(r); }
template <typename Index, typename Function>
    requires std::is_integral_v<Index>
void parallel_for(Index first, Index last, const Function& f) {
    for (Index i = first; i < last; ++i) f(i);
}

template <typename Range, typename Value, typename RealBody, typename Reduction>
Value parallel_reduce(const Range& r, const Value& identity, const RealBody& body, const Reduction&) {
    return body(r, identity);
}
template <typename Range, typename Value, typename RealBody, typename Reduction, typename P>
Value parallel_reduce(const Range& r, const Value& identity, const RealBody& body, const Reduction&, P&&) {
    return body(r, identity);
}
template <typename Range, typename Body>
void parallel_reduce(const Range& r, Body& body) { body(r); }
template <typename Range, typename Body>
void parallel_deterministic_reduce(const Range& r, Body& body) { body(r); }
template <typename Range, typename Value, typename RealBody, typename Reduction>
Value parallel_deterministic_reduce(const Range& r, const Value& identity, const RealBody& body, const Reduction&) {
    return body(r, identity);
}

template <typename It>
void parallel_sort(It b, It e) { std::sort(b, e); }
template <typename It, typename Cmp>
void parallel_sort(It b, It e, const Cmp& c) { std::sort(b, e, c); }

template <typename T>
class enumerable_thread_specific {
public:
    using iterator = typename std::list<T>::iterator;
    using const_iterator = typename std::list<T>::const_iterator;
    enumerable_thread_specific() = default;
    explicit enumerable_thread_specific(const T& init) : init_(init), hasInit_(true) {}
    template <typename F>
        requires std::is_invocable_r_v<T, F>
    explicit enumerable_thread_specific(F f) : init_(f()), hasInit_(true) {}
    T& local() {
        if (items_.empty()) items_.push_back(hasInit_ ? init_ : T{});
        return items_.front();
    }
    T& local(bool& exists) {
        exists = !items_.empty();
        return local();
    }
    iterator begin() { return items_.begin(); }
    iterator end() { return items_.end(); }
    const_iterator begin() const { return items_.begin(); }
    const_iterator end() const { return items_.end(); }
    std::size_t size() const { return items_.size(); }
    bool empty() const { return items_.empty(); }
    void clear() { items_.clear(); }
    template <typename F>
    void combine_each(F f) { for (auto& x : items_) f(x); }
    template <typename F>
    T combine(F f) {
        if (items_.empty()) return hasInit_ ? init_ : T{};
        auto it = items_.begin();
        T acc = *it;
        for (++it; it != items_.end(); ++it) acc = f(acc, *it);
        return acc;
    }

private:
    std::list<T> items_;
    T init_{};
    bool hasInit_ = false;
};

class task_group {
public:
    template <typename F>
    void run(F&& f) { f(); }
    template <typename F>
    void run_and_wait(F&& f) { f(); }
    void wait() {}
};

class task_arena {
public:
    static constexpr int automatic = -1;
    task_arena(int = automatic, unsigned = 1) {}
    template <typename F>
    auto execute(F&& f) { return f(); }
    int max_concurrency() const { return 1; }
};

namespace this_task_arena {
inline int current_thread_index() { return 0; }
inline int max_concurrency() { return 1; }
template <typename F>
auto isolate(F&& f) { return f(); }
}  // namespace this_task_arena

class global_control {
public:
    enum parameter { max_allowed_parallelism, thread_stack_size };
    global_control(parameter, std::size_t) {}
    static std::size_t active_value(parameter p) { return p == max_allowed_parallelism ? 1 : 0; }
};

class task_scheduler_observer {
public:
    virtual ~task_scheduler_observer() = default;
    void observe(bool = true) {}
    virtual void on_scheduler_entry(bool) {}
    virtual void on_scheduler_exit(bool) {}
};

class spin_mutex {
public:
    void lock() {}
    void unlock() {}
    bool try_lock() { return true; }
    class scoped_lock {
    public:
        scoped_lock() = default;
        explicit scoped_lock(spin_mutex&) {}
        void acquire(spin_mutex&) {}
        void release() {}
    };
};
using mutex = spin_mutex;

}  // namespace tbb

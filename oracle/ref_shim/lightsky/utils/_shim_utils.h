/*
 * Compatibility shim for LightSky's "utils" library (an absent submodule of
 * the reference tree), written for building the reference's draw-path
 * sources as a CPU oracle: aligned allocation and owning pointers, memory
 * fill/copy, a stable LSD radix sort, a task worker thread, assertions and
 * logging. Only what those sources use is provided.
 */
#ifndef LS_SHIM_UTILS_H
#define LS_SHIM_UTILS_H

#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "../setup/_shim_setup.h"

#define LS_ASSERT(x) do { if (!(x)) { std::fprintf(stderr, "assertion failed: %s (%s:%d)\n", #x, __FILE__, __LINE__); std::abort(); } } while (0)
#define LS_DEBUG_ASSERT(x) do { (void)sizeof(x); } while (0)
#define LS_LOG_MSG(...) do { } while (0)
#define LS_LOG_ERR(...) do { } while (0)

namespace ls
{
namespace utils
{

/* string hash for SL_Animation's ids: FNV-1a, 64 bits */
typedef uint64_t hash_t;
inline hash_t string_hash(const char* str) noexcept
{
    hash_t h = 14695981039346656037ull;
    for (; *str; ++str) h = (h ^ (uint8_t)*str) * 1099511628211ull;
    return h;
}


inline void* aligned_malloc(std::size_t n) noexcept
{
    void* p = nullptr;
    if (posix_memalign(&p, 64, n ? n : 64) != 0) return nullptr;
    return p;
}

inline void aligned_free(void* p) noexcept { std::free(p); }

struct AlignedDeleter
{
    void operator()(void* p) const noexcept { aligned_free(p); }
};

template <typename T> struct AlignedArrayDeleter
{
    std::size_t count = 0;
    void operator()(T* p) const noexcept
    {
        if (!p) return;
        for (std::size_t i = 0; i < count; ++i) p[i].~T();
        aligned_free(p);
    }
};

template <typename T> struct AlignedPointerDeleter
{
    void operator()(T* p) const noexcept
    {
        if (!p) return;
        p->~T();
        aligned_free(p);
    }
};

template <typename T, typename D = std::default_delete<T>>
using Pointer = std::unique_ptr<T, D>;

/* std allocator returning 64-byte aligned storage */
template <typename T>
struct AlignedAllocator
{
    typedef T value_type;
    AlignedAllocator() noexcept = default;
    template <typename U> AlignedAllocator(const AlignedAllocator<U>&) noexcept {}
    T* allocate(std::size_t n)
    {
        void* p = aligned_malloc(sizeof(T) * n);
        if (!p) throw std::bad_alloc();
        return static_cast<T*>(p);
    }
    void deallocate(T* p, std::size_t) noexcept { aligned_free(p); }
    template <typename U> bool operator==(const AlignedAllocator<U>&) const noexcept { return true; }
    template <typename U> bool operator!=(const AlignedAllocator<U>&) const noexcept { return false; }
};

template <typename T>
using UniqueAlignedArray = std::unique_ptr<T[], AlignedArrayDeleter<T>>;

template <typename T>
using UniqueAlignedPointer = std::unique_ptr<T, AlignedPointerDeleter<T>>;

template <typename T>
inline UniqueAlignedArray<T> make_unique_aligned_array(std::size_t n) noexcept
{
    T* p = static_cast<T*>(aligned_malloc(sizeof(T) * (n ? n : 1)));
    for (std::size_t i = 0; i < n; ++i) new (&p[i]) T();
    AlignedArrayDeleter<T> d;
    d.count = n;
    return UniqueAlignedArray<T>(p, d);
}

template <typename T, typename... Args>
inline UniqueAlignedPointer<T> make_unique_aligned_pointer(Args&&... args) noexcept
{
    T* p = static_cast<T*>(aligned_malloc(sizeof(T)));
    new (p) T(std::forward<Args>(args)...);
    return UniqueAlignedPointer<T>(p);
}

inline void fast_memset(void* dst, int v, std::size_t numBytes) noexcept { std::memset(dst, v, numBytes); }
inline void fast_memcpy(void* dst, const void* src, std::size_t numBytes) noexcept { std::memcpy(dst, src, numBytes); }
template <typename T> inline void fast_copy(T* dst, const T* src, std::size_t count) noexcept { for (std::size_t i = 0; i < count; ++i) dst[i] = src[i]; }

template <typename T> inline void fill_pattern(void* dst, T v, std::size_t numBytes) noexcept
{
    unsigned char* p = static_cast<unsigned char*>(dst);
    std::size_t i = 0;
    for (; i + sizeof(T) <= numBytes; i += sizeof(T)) std::memcpy(p + i, &v, sizeof(T));
    if (i < numBytes) std::memcpy(p + i, &v, numBytes - i);
}
inline void fast_memset_2(void* dst, uint16_t v, std::size_t numBytes) noexcept { fill_pattern<uint16_t>(dst, v, numBytes); }
inline void fast_memset_4(void* dst, uint32_t v, std::size_t numBytes) noexcept { fill_pattern<uint32_t>(dst, v, numBytes); }
inline void fast_memset_8(void* dst, uint64_t v, std::size_t numBytes) noexcept { fill_pattern<uint64_t>(dst, v, numBytes); }

template <typename T> inline void fast_fill(T* dst, const T& v, std::size_t count) noexcept
{
    for (std::size_t i = 0; i < count; ++i) dst[i] = v;
}

/* Stable least-significant-digit radix sort of n items by a 64-bit key,
 * result left in `items`. */
template <typename T, typename KeyFn>
inline void sort_radix(T* items, T* temp, uint64_t n, const KeyFn& key) noexcept
{
    if (n < 2) return;
    uint64_t maxKey = 0;
    for (uint64_t i = 0; i < n; ++i) maxKey |= (uint64_t)key(items[i]);
    T* src = items;
    T* dst = temp;
    for (unsigned shift = 0; shift < 64 && (maxKey >> shift); shift += 8)
    {
        std::size_t count[257] = {0};
        for (uint64_t i = 0; i < n; ++i) ++count[(((uint64_t)key(src[i])) >> shift & 0xFF) + 1];
        for (int b = 0; b < 256; ++b) count[b + 1] += count[b];
        for (uint64_t i = 0; i < n; ++i) dst[count[((uint64_t)key(src[i])) >> shift & 0xFF]++] = src[i];
        T* t = src; src = dst; dst = t;
    }
    if (src != items) for (uint64_t i = 0; i < n; ++i) items[i] = src[i];
}

inline std::thread::id get_thread_id() noexcept { return std::this_thread::get_id(); }
inline void set_thread_affinity(std::thread::id, unsigned) noexcept {}

/* A thread that runs pushed copies of a task when flushed. */
template <typename TaskType>
class WorkerThread
{
  public:
    explicit WorkerThread(std::size_t = 0) : mStop(false), mBusy(false), mPending(false)
    {
        mThread = std::thread([this]() { run(); });
    }

    ~WorkerThread()
    {
        {
            std::lock_guard<std::mutex> g(mLock);
            mStop = true;
        }
        mCond.notify_all();
        if (mThread.joinable()) mThread.join();
    }

    void busy_waiting(bool) noexcept {}

    void push(const TaskType& t)
    {
        std::lock_guard<std::mutex> g(mLock);
        mQueue.push_back(t);
    }

    void flush()
    {
        {
            std::lock_guard<std::mutex> g(mLock);
            mPending = !mQueue.empty();
        }
        mCond.notify_all();
    }

    bool ready()
    {
        std::lock_guard<std::mutex> g(mLock);
        return !mPending && !mBusy;
    }

    void wait()
    {
        std::unique_lock<std::mutex> g(mLock);
        mDone.wait(g, [this]() { return !mPending && !mBusy; });
    }

  private:
    void run()
    {
        for (;;)
        {
            std::vector<TaskType> work;
            {
                std::unique_lock<std::mutex> g(mLock);
                mCond.wait(g, [this]() { return mStop || mPending; });
                if (mStop) return;
                work.swap(mQueue);
                mPending = false;
                mBusy = true;
            }
            for (TaskType& t : work) t();
            {
                std::lock_guard<std::mutex> g(mLock);
                mBusy = false;
            }
            mDone.notify_all();
        }
    }

    std::mutex mLock;
    std::condition_variable mCond, mDone;
    std::vector<TaskType> mQueue;
    bool mStop, mBusy, mPending;
    std::thread mThread;
};

/* Declared for SL_VertexCache (compiled out by SL_VERTEX_CACHING_ENABLED 0). */
template <typename T, std::size_t N>
class IndexedCache
{
  public:
    template <typename F> const T& query_or_update(std::size_t key, const F& f) noexcept { f(key, mVal); return mVal; }
  private:
    T mVal;
};

template <typename T, std::size_t N> using LRUCache = IndexedCache<T, N>;
template <typename T> using LRU8WayCache = IndexedCache<T, 8>;

} // namespace utils
} // namespace ls

#endif

// Host emulation of the warp intrinsics the ant kernel uses, so that the
// kernel's own source runs on the CPU: one OS thread per lane, every warp
// intrinsic a barrier-synchronised exchange between the 32 threads, and
// lanes delayed at random before each barrier so that code which relies on
// lanes running in lockstep between synchronisation points (a read of
// shared state that another lane writes without a __syncwarp between them)
// gives different values in different lanes.  A barrier that waits more than
// 20 seconds reports every lane's last call site (a warp intrinsic reached
// by some lanes only) and aborts.  Test infrastructure only.
#pragma once
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

#define __device__
#define __host__
#define __forceinline__ inline
#define __global__
#define __launch_bounds__(...)
#define __shared__
#define __align__(x) alignas(x)

struct int2 { int x, y; };
inline int2 make_int2(int x, int y) { return {x, y}; }
struct uint2 { unsigned x, y; };
struct uint4 { unsigned x, y, z, w; };
struct float4 { float x, y, z, w; };
typedef int cudaError_t;
typedef void* cudaStream_t;

#include <random>
#include <thread>
inline void jitter() {
    thread_local std::minstd_rand rng(std::hash<std::thread::id>{}(std::this_thread::get_id()));
    const unsigned r = rng() % 100;
    if (r < 3) std::this_thread::sleep_for(std::chrono::microseconds(rng() % 200));
    else if (r < 20) std::this_thread::yield();
}
struct Warp {
    std::mutex mu;
    std::condition_variable cv;
    int arrived = 0;
    unsigned long long generation = 0;
    unsigned long long slot[32];
    int site[32];
    void wait(unsigned lane, int line) {
        jitter();
        std::unique_lock<std::mutex> lk(mu);
        site[lane] = line;
        const unsigned long long gen = generation;
        if (++arrived == 32) {
            arrived = 0;
            ++generation;
            cv.notify_all();
            return;
        }
        if (!cv.wait_for(lk, std::chrono::seconds(20), [&] { return generation != gen; })) {
            std::fprintf(stderr, "WARP HANG: lane %u at line %d; sites:", lane, line);
            for (int i = 0; i < 32; ++i) std::fprintf(stderr, " %d", site[i]);
            std::fprintf(stderr, "\n");
            std::fflush(stderr);
            std::abort();
        }
    }
};
extern thread_local Warp* tl_warp;
extern thread_local unsigned tl_lane;

template <class T> inline unsigned long long to_bits(T v) { unsigned long long b = 0; std::memcpy(&b, &v, sizeof(T)); return b; }
template <class T> inline T from_bits(unsigned long long b) { T v; std::memcpy(&v, &b, sizeof(T)); return v; }

template <class T> inline T emu_exch(int line, T v, unsigned src) {
    Warp* w = tl_warp;
    w->slot[tl_lane] = to_bits(v);
    w->wait(tl_lane, line);
    T r = from_bits<T>(w->slot[src & 31]);
    w->wait(tl_lane, line);
    return r;
}
template <class T> inline T emu_shfl(int line, unsigned, T v, int src) { return emu_exch(line, v, (unsigned)src); }
template <class T> inline T emu_shfl_up(int line, unsigned, T v, unsigned d) {
    const int s = (int)tl_lane - (int)d;
    return emu_exch(line, v, s < 0 ? tl_lane : (unsigned)s);
}
template <class T> inline T emu_shfl_xor(int line, unsigned, T v, int m) { return emu_exch(line, v, tl_lane ^ (unsigned)m); }
inline void emu_syncwarp(int line) { tl_warp->wait(tl_lane, line); }
inline unsigned emu_ballot(int line, unsigned, int p) {
    Warp* w = tl_warp;
    w->slot[tl_lane] = p ? 1 : 0;
    w->wait(tl_lane, line);
    unsigned m = 0;
    for (int i = 0; i < 32; ++i) m |= (unsigned)(w->slot[i] & 1) << i;
    w->wait(tl_lane, line);
    return m;
}
template <class T, class F> inline T emu_reduce(int line, T v, F f) {
    Warp* w = tl_warp;
    w->slot[tl_lane] = to_bits(v);
    w->wait(tl_lane, line);
    T r = from_bits<T>(w->slot[0]);
    for (int i = 1; i < 32; ++i) r = f(r, from_bits<T>(w->slot[i]));
    w->wait(tl_lane, line);
    return r;
}
inline unsigned emu_radd(int line, unsigned v) { return emu_reduce(line, v, [](unsigned a, unsigned b) { return a + b; }); }
inline int emu_radd(int line, int v) { return emu_reduce(line, v, [](int a, int b) { return a + b; }); }
inline int emu_rmax(int line, int v) { return emu_reduce(line, v, [](int a, int b) { return a > b ? a : b; }); }
inline unsigned emu_rmin(int line, unsigned v) { return emu_reduce(line, v, [](unsigned a, unsigned b) { return a < b ? a : b; }); }

#define __shfl_sync(m, v, s) emu_shfl(__LINE__, m, v, s)
#define __shfl_up_sync(m, v, d) emu_shfl_up(__LINE__, m, v, d)
#define __shfl_xor_sync(m, v, x) emu_shfl_xor(__LINE__, m, v, x)
#define __syncwarp(...) emu_syncwarp(__LINE__)
#define __ballot_sync(m, p) emu_ballot(__LINE__, m, p)
#define __any_sync(m, p) (emu_ballot(__LINE__, m, p) != 0)
#define __reduce_add_sync(m, v) emu_radd(__LINE__, v)
#define __reduce_max_sync(m, v) emu_rmax(__LINE__, v)
#define __reduce_min_sync(m, v) emu_rmin(__LINE__, v)

inline unsigned __umulhi(unsigned a, unsigned b) { return (unsigned)(((unsigned long long)a * b) >> 32); }
inline float __uint2float_rn(unsigned v) { return (float)v; }
inline int __float2int_rn(float f) { return (int)std::nearbyint(f); }
inline int __ffs(unsigned v) { return __builtin_ffs((int)v); }
inline int __ffs(int v) { return __builtin_ffs(v); }
inline int __popc(unsigned v) { return __builtin_popcount(v); }
inline int __clz(unsigned v) { return v ? __builtin_clz(v) : 32; }
template <class T> inline T __ldg(const T* p) { return *p; }
extern std::mutex g_atomic;
inline unsigned atomicOr(unsigned* p, unsigned v) { std::lock_guard<std::mutex> g(g_atomic); unsigned o = *p; *p = o | v; return o; }

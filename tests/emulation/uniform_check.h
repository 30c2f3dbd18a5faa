// Checks, after every construction step of the emulated ant kernel, that the
// per-ant values every lane keeps in its own registers (current node, step
// and MNE counters, tour length, relocation run, checklist) agree across the
// 32 lanes; a difference is a warp race and aborts the emulation.
#pragma once
namespace faco {
inline void uniform_check(const char* where, unsigned cur, unsigned steps, unsigned mne, long long cost, unsigned m,
                          unsigned p, unsigned t, unsigned dir, unsigned pending, unsigned tail) {
    const unsigned long long v[10] = {cur, steps, mne, (unsigned long long)cost, m, p, t, dir, pending, tail};
    bool bad = false;
    int which = -1;
    for (int i = 0; i < 10; ++i)
        if (__shfl_sync(kFull, v[i], 0) != v[i]) { bad = true; which = i; }
    if (__any_sync(kFull, bad)) {
        if (bad) std::fprintf(stderr, "lanes disagree after a %s step: lane %u, value %d\n", where, tl_lane, which);
        std::fflush(stderr);
        __syncwarp();
        std::abort();
    }
}
}  // namespace faco

// CPU check of fk::FirstFit (the request server's device-block bookkeeping):
// a seeded random sequence of allocations and releases against a plain model
// of the block, one byte-granular flag per 256-byte unit.  Exits non-zero
// with a message at the first disagreement.
#include <cstdint>
#include <cstdio>
#include <vector>

#include "fk_firstfit.h"

namespace {

struct Lcg {
    uint64_t s;
    uint64_t next() {
        s = s * 6364136223846793005ull + 1442695040888963407ull;
        return s >> 33;
    }
};

int fail(const char* what, long step) {
    std::printf("FAIL step %ld: %s\n", step, what);
    return 1;
}

}  // namespace

int main() {
    const size_t unit = 256;
    for (uint64_t seed = 1; seed <= 20; ++seed) {
        Lcg rng{seed};
        const size_t cap_units = 64 + rng.next() % 512;
        fk::FirstFit ff;
        ff.reset(cap_units * unit - (rng.next() % unit));  // rounded up to cap_units units
        if (ff.capacity() != cap_units * unit) return fail("capacity not rounded to 256", -1);
        std::vector<int> owner(cap_units, -1);  // live block id per unit
        struct Live { size_t off, units; };
        std::vector<Live> live;
        size_t in_use = 0, peak = 0;
        for (long step = 0; step < 4000; ++step) {
            const bool do_alloc = live.empty() || rng.next() % 100 < 55;
            if (do_alloc) {
                const size_t bytes = 1 + rng.next() % (unit * 24);
                const size_t units = (bytes + unit - 1) / unit;
                // first fit in the model: the lowest run of `units` free units
                size_t want = fk::FirstFit::NONE, run = 0;
                for (size_t i = 0; i < cap_units; ++i) {
                    run = owner[i] < 0 ? run + 1 : 0;
                    // a free range of the allocator is a maximal run; first fit takes the
                    // lowest maximal run long enough, at its start
                    if (run == units) {
                        size_t start = i + 1 - units;
                        while (start > 0 && owner[start - 1] < 0) --start;
                        want = start * unit;
                        break;
                    }
                }
                const size_t got = ff.alloc(bytes);
                if (got != want) return fail("alloc differs from first fit", step);
                if (got == fk::FirstFit::NONE) continue;
                if (got % unit) return fail("offset not 256-aligned", step);
                for (size_t i = got / unit; i < got / unit + units; ++i) {
                    if (owner[i] >= 0) return fail("overlap with a live block", step);
                    owner[i] = (int)live.size();
                }
                live.push_back({got, units});
                in_use += units * unit;
                if (in_use > peak) peak = in_use;
            } else {
                const size_t k = rng.next() % live.size();
                const Live b = live[k];
                ff.release(b.off);
                for (size_t i = b.off / unit; i < b.off / unit + b.units; ++i) owner[i] = -1;
                live[k] = live.back();
                live.pop_back();
                for (size_t j = 0; j < live.size(); ++j)
                    for (size_t i = live[j].off / unit; i < live[j].off / unit + live[j].units; ++i) owner[i] = (int)j;
                in_use -= b.units * unit;
                // a release of an offset that is not a block start is ignored
                if (b.units > 1) ff.release(b.off + unit);
            }
            if (ff.in_use() != in_use) return fail("in_use differs", step);
            if (ff.peak() != peak) return fail("peak differs", step);
            // the free ranges are exactly the maximal runs of free units
            size_t runs = 0, largest = 0, run = 0;
            for (size_t i = 0; i <= cap_units; ++i) {
                if (i < cap_units && owner[i] < 0) {
                    ++run;
                } else if (run) {
                    ++runs;
                    if (run * unit > largest) largest = run * unit;
                    run = 0;
                }
            }
            if (ff.free_ranges() != runs) return fail("free ranges not coalesced", step);
            if (ff.largest_free() != largest) return fail("largest free range differs", step);
        }
        for (const Live& b : live) ff.release(b.off);
        if (ff.in_use() != 0 || ff.free_ranges() != 1 || ff.largest_free() != ff.capacity())
            return fail("block not whole after releasing everything", -2);
    }
    std::printf("ok\n");
    return 0;
}

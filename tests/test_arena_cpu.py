"""The batch engine's arena free list (das_gb300/csrc/arena.h), compiled with g++ and
driven on the host: a seeded random sequence of allocations and frees, with every
invariant checked after each operation (aligned offsets inside the arena, no live block
overlapping another or a free block, free plus live bytes equal to the arena, free
blocks coalesced), first fit, and the whole arena one block again once everything is
freed."""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DRIVER = r"""
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "arena.h"

struct Live { size_t off, bytes; };

static unsigned long long state = 12345;
static unsigned long long rnd() { state = state * 6364136223846793005ULL + 1442695040888963407ULL;
                                  return state >> 33; }
#define CHECK(c) do { if (!(c)) { std::printf("FAIL %s line %d op %d\n", #c, __LINE__, op); \
                                  return 1; } } while (0)

int main()
{
    const size_t align = 256, arena = 1000 * align + 100;  // not a multiple: rounded down
    w2d::ArenaFreeList fl(align);
    fl.reset(arena);
    const size_t usable = arena / align * align;
    std::vector<Live> live;
    int op = 0;
    CHECK(fl.blocks().size() == 1 && fl.largest() == usable);
    for (op = 0; op < 20000; ++op) {
        if (live.empty() || rnd() % 100 < 55) {
            const size_t want = 1 + rnd() % (40 * align);
            size_t off = 0;
            const size_t lowest_fit = [&] {
                for (const auto& kv : fl.blocks())
                    if (kv.second >= fl.round(want)) return kv.first;
                return (size_t)-1;
            }();
            const bool ok = fl.alloc(want, &off);
            CHECK(ok == (lowest_fit != (size_t)-1));
            if (ok) {
                CHECK(off == lowest_fit);  // first fit
                CHECK(off % align == 0 && off + fl.round(want) <= usable);
                for (const auto& l : live)
                    CHECK(off + fl.round(want) <= l.off || l.off + fl.round(l.bytes) <= off);
                live.push_back({off, want});
            }
        } else {
            const size_t i = rnd() % live.size();
            fl.free(live[i].off, live[i].bytes);
            live.erase(live.begin() + (long)i);
        }
        size_t free_bytes = 0, prev_end = 0;
        bool first = true;
        for (const auto& kv : fl.blocks()) {
            CHECK(kv.second > 0 && kv.first % align == 0 && kv.second % align == 0);
            CHECK(first || kv.first > prev_end);  // sorted, disjoint, never adjacent
            prev_end = kv.first + kv.second;
            first = false;
            free_bytes += kv.second;
            for (const auto& l : live)
                CHECK(kv.first + kv.second <= l.off || l.off + fl.round(l.bytes) <= kv.first);
        }
        size_t live_bytes = 0;
        for (const auto& l : live) live_bytes += fl.round(l.bytes);
        CHECK(free_bytes + live_bytes == usable);
    }
    for (const auto& l : live) fl.free(l.off, l.bytes);
    CHECK(fl.blocks().size() == 1 && fl.blocks().begin()->first == 0 &&
          fl.blocks().begin()->second == usable);
    std::printf("OK %d operations\n", op);
    return 0;
}
"""


def test_arena_free_list(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    src = tmp_path / "arena_driver.cpp"
    src.write_text(DRIVER)
    exe = tmp_path / "arena_driver"
    inc = os.path.join(REPO, "das_gb300", "csrc")
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-I", inc, str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.startswith("OK"), r.stdout + r.stderr

"""The per-device cache of one-time kernel set-up (csrc/per_device.h), run on
the CPU with a fake device ordinal and a fake set-up function.

A kernel's dynamic-shared-memory attribute and its persistent grid size belong
to one device: the cache must run the set-up once for every device a process
uses, keep each device's own value, retry after a failed set-up, and reject
ordinals it cannot hold.  No GPU is involved: the header is plain C++."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "fft-ocean-waves_gb300", "csrc")

PROGRAM = r"""
#include <cstdio>
#include <thread>
#include <vector>
#include "per_device.h"

static std::atomic<int> g_calls[ocean::kMaxDevices];
static int g_fail_once[ocean::kMaxDevices];

// stands in for cudaFuncSetAttribute + occupancy on device `dev`: its value
// differs per device (e.g. SMs x CTAs per SM)
static int fake_setup(int dev, int* v)
{
    g_calls[dev].fetch_add(1);
    if (g_fail_once[dev]) { g_fail_once[dev] = 0; return 7; }
    *v = 100 + dev;
    return 0;
}

int main()
{
    ocean::PerDevice cache;
    int bad = 0;
    // devices 0..3 in turn, then again: set-up runs once per device, values stay per device
    for (int round = 0; round < 3; ++round)
        for (int dev = 0; dev < 4; ++dev) {
            int v = 0;
            int rc = cache.get(dev, &v, -1, [&](int* out) { return fake_setup(dev, out); });
            if (rc != 0 || v != 100 + dev) { std::printf("bad value dev %d: rc %d v %d\n", dev, rc, v); bad = 1; }
        }
    for (int dev = 0; dev < 4; ++dev)
        if (g_calls[dev].load() != 1) { std::printf("dev %d set up %d times\n", dev, g_calls[dev].load()); bad = 1; }
    // a failed set-up returns its error and is retried by the next call
    g_fail_once[9] = 1;
    int v = 0;
    int rc = cache.get(9, &v, -1, [&](int* out) { return fake_setup(9, out); });
    if (rc != 7) { std::printf("failed set-up returned %d\n", rc); bad = 1; }
    rc = cache.get(9, &v, -1, [&](int* out) { return fake_setup(9, out); });
    if (rc != 0 || v != 109 || g_calls[9].load() != 2) { std::printf("retry: rc %d v %d\n", rc, v); bad = 1; }
    // ordinals outside the table
    for (int dev : {-1, ocean::kMaxDevices, 1000}) {
        rc = cache.get(dev, &v, -1, [&](int* out) { *out = 1; return 0; });
        if (rc != -1) { std::printf("ordinal %d accepted\n", dev); bad = 1; }
    }
    // threads driving devices 20..27 concurrently: each sees its own device's value
    std::vector<std::thread> th;
    std::atomic<int> wrong{0};
    for (int k = 0; k < 32; ++k)
        th.emplace_back([&, k] {
            const int dev = 20 + k % 8;
            for (int i = 0; i < 1000; ++i) {
                int w = 0;
                if (cache.get(dev, &w, -1, [&](int* out) { return fake_setup(dev, out); }) != 0 || w != 100 + dev)
                    wrong.fetch_add(1);
            }
        });
    for (auto& t : th) t.join();
    if (wrong.load()) { std::printf("%d wrong lookups under threads\n", wrong.load()); bad = 1; }
    for (int dev = 20; dev < 28; ++dev)
        if (g_calls[dev].load() < 1 || g_calls[dev].load() > 4) { std::printf("dev %d: %d set-ups\n", dev, g_calls[dev].load()); bad = 1; }
    std::printf(bad ? "FAIL\n" : "OK\n");
    return bad;
}
"""


def test_per_device_cache(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "per_device_test.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "per_device_test"
    subprocess.check_call([cxx, "-std=c++17", "-O1", "-pthread", "-I", CSRC, str(src), "-o", str(exe)])
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout + r.stderr


def test_launchers_use_the_per_device_cache():
    """No launcher sets a kernel attribute or queries occupancy on its own:
    both go through launch_setup.cuh's per-device helpers."""
    for name in os.listdir(CSRC):
        if not name.endswith((".cu", ".cpp")):
            continue
        src = open(os.path.join(CSRC, name)).read()
        assert "cudaFuncSetAttribute" not in src, name
        assert "cudaOccupancyMaxActiveBlocksPerMultiprocessor" not in src, name
    assert "PerDevice" in open(os.path.join(CSRC, "launch_setup.cuh")).read()

"""Per-device bookkeeping of the walker kernel's attributes (CPU only).

cudaFuncSetAttribute acts on the current device, so the library records the
dynamic shared-memory size each kernel has been opted into per device
(``csrc/dmc_attr.h``).  This test compiles a small C++ driver against that
header with g++ and a fake set function: a second device must get its own
set call, a smaller size on a device already set must not call again, a
failed set must not be recorded, and host threads setting different devices
at the same time must each end with their own record.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "dmcbcs_project_gb300", "csrc")

DRIVER = r"""
#include <atomic>
#include <cstdio>
#include <thread>
#include <vector>
#include "dmc_attr.h"

int main()
{
    dmc::AttrCache c;
    std::atomic<int> calls{0};
    auto ok = [&](int) { ++calls; return 0; };
    auto bad = [&](int) { ++calls; return 7; };
    // device 0 set to 1000, then 500 needs nothing, 2000 needs a call
    if (c.ensure(0, 1, 1000, ok) != 0 || calls != 1) return 1;
    if (c.ensure(0, 1, 500, ok) != 0 || calls != 1) return 2;
    if (c.ensure(0, 1, 2000, ok) != 0 || calls != 2 || c.recorded(0, 1) != 2000) return 3;
    // device 1 is independent of device 0
    if (c.recorded(1, 1) != -1) return 4;
    if (c.ensure(1, 1, 1000, ok) != 0 || calls != 3 || c.recorded(1, 1) != 1000) return 5;
    // a failed set is returned and not recorded
    if (c.ensure(2, 1, 100, bad) != 7 || c.recorded(2, 1) != -1) return 6;
    // out-of-table devices are never cached
    calls = 0;
    c.ensure(dmc::AttrCache::kMaxDevices, 1, 10, ok);
    c.ensure(dmc::AttrCache::kMaxDevices, 1, 10, ok);
    if (calls != 2) return 7;
    // concurrent host threads, one device each, growing sizes
    std::vector<std::thread> th;
    std::atomic<int> setc{0};
    for (int d = 3; d < 11; ++d)
        th.emplace_back([&, d] {
            for (int v = 1; v <= 2000; ++v) c.ensure(d, 2, v / 10, [&](int) { ++setc; return 0; });
        });
    for (auto& t : th) t.join();
    for (int d = 3; d < 11; ++d)
        if (c.recorded(d, 2) != 200) return 8;
    if (setc != 8 * 201) return 9;   // sizes 0..200 once each per device
    std::puts("ok");
    return 0;
}
"""


def test_attr_cache_per_device(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    src = tmp_path / "attr_driver.cpp"
    exe = tmp_path / "attr_driver"
    src.write_text(DRIVER)
    subprocess.run([gxx, "-std=c++17", "-O1", "-pthread", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", (r.returncode, r.stdout, r.stderr)

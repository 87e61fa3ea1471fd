"""The kw::Pricer subclasses that INTEGRATION.md gives a maintainer of the reference
(Fd1dGpu_Pricer, Fd1dBsGpu_Pricer) compile verbatim against the reference's own
headers (src/Pricer/kwPricer.h, src/Core/kwConfig.h), link against libkwg.so and
run: init() succeeds on a GPU and reports the missing device without one.  Skipped
where the reference sources are absent."""
import os
import re
import shutil
import subprocess
import sys

import pytest

from conftest import ROOT

MAIN = r"""
#include <cstdio>
int main() {
    kw::Config config;
    config.set("FD1D.X_GRID_SIZE", "64");
    config.set("FD1D.T_GRID_SIZE", "32");
    kw::Fd1dBsGpu_Pricer pricer;
    const kw::Error e = pricer.init(config);
    std::printf("init: [%s]\n", e.c_str());
    return 0;
}
"""


def test_integration_pricers_compile_link_and_run(built, tmp_path):
    import kwg

    sys.path.insert(0, ROOT)
    import __graft_entry__ as ge

    if not os.path.isdir(ge.REF_SRC):
        pytest.skip("reference sources absent")
    if not shutil.which("g++"):
        pytest.skip("no g++")
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```cpp\n(.*?)```", text, re.S)
    assert len(blocks) >= 2
    src = tmp_path / "pricers.cpp"
    src.write_text("\n".join(blocks[:2]) + MAIN)
    exe = tmp_path / "pricers"
    lib_dir = os.path.dirname(kwg.LIB_PATH)
    subprocess.run(["g++", "-std=c++20", "-I", ge.REF_SRC, "-I", os.path.join(ROOT, "include"), str(src),
                    "-L", lib_dir, "-lkwg", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() in ("init: []", "init: [Fd1dGpu_Pricer::init: no CUDA device]"), out.stdout

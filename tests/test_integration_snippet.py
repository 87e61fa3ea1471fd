"""The kw::Pricer subclasses the integration guide gives a maintainer of the reference
(Fd1dGpu_Pricer, Fd1dBsGpu_Pricer), compiled verbatim from the guide, linked against
libkwg.so and run.

* Against the reference's own headers (src/Pricer/kwPricer.h, src/Core/kwConfig.h):
  init() succeeds on a GPU and reports the missing device without one.  Skipped
  where the reference sources are absent.
* Against tests/kw_pricer_api, a stand-in for those headers written for these tests
  (same signatures: src/Pricer/kwPricer.h:12-22, src/Core/kwConfig.h:21-73), which
  travels with the repository: init() on CPU, and on the GPU price() itself --
  the 12-option table of test/kwPricer_test.cpp:16-28 and the 6000-option QdFp
  portfolio of test/kwPortfolio_test.cpp:41-56, through both classes, against the
  reference's own prices (golden fixtures) or the oracle, to 1e-10 relative."""
import os
import re
import shutil
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, golden

STANDIN = os.path.join(ROOT, "tests", "kw_pricer_api")
REL_TOL = 1e-10
PRICE_FLOOR = 1e-12
# FD1D-BS prices are differences of FD prices of tens of currency units; below this
# floor they are compared absolutely, to REL_TOL * BS_PRICE_FLOOR = 1e-13, as in
# tests/test_fd1d_bs_gpu.py
BS_PRICE_FLOOR = 1e-3

INIT_MAIN = r"""
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

# Prices a file of 56-byte kw::Option records through one of the two classes:
#   pricers MODE X_DIM T_DIM SCALE DENSITY IN OUT      (MODE: FD1D or FD1D-BS)
PRICE_MAIN = r"""
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
int main(int argc, char** argv) {
    if (argc != 8) return 2;
    kw::Config config;
    config.set("FD1D.X_GRID_SIZE", (long long)std::atoll(argv[2]));
    config.set("FD1D.T_GRID_SIZE", (long long)std::atoll(argv[3]));
    config.set("FD1D.SCALE", std::atof(argv[4]));
    config.set("FD1D.DENSITY", std::atof(argv[5]));
    std::unique_ptr<kw::Pricer> pricer;
    if (std::strcmp(argv[1], "FD1D-BS") == 0) pricer = std::make_unique<kw::Fd1dBsGpu_Pricer>();
    else pricer = std::make_unique<kw::Fd1dGpu_Pricer>();
    kw::Error e = pricer->init(config);
    if (!e.empty()) { std::printf("init: [%s]\n", e.c_str()); return 3; }
    std::FILE* f = std::fopen(argv[6], "rb");
    if (!f) return 4;
    std::vector<kw::Option> assets;
    kw::Option o;
    while (std::fread(&o, sizeof o, 1, f) == 1) assets.push_back(o);
    std::fclose(f);
    std::vector<double> prices;
    e = pricer->price(assets, prices);
    std::printf("price: [%s] %zu\n", e.c_str(), prices.size());
    if (!e.empty()) return 5;
    f = std::fopen(argv[7], "wb");
    if (!f) return 4;
    std::fwrite(prices.data(), sizeof(double), prices.size(), f);
    std::fclose(f);
    return 0;
}
"""


def _env():
    """Loader path for libcudart beside the CUDA toolkit that built libkwg.so."""
    env = dict(os.environ)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cuda = os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    libs = [os.path.join(cuda, "lib64")] + [os.path.join(cuda, "targets", t, "lib")
                                            for t in ("sbsa-linux", "aarch64-linux", "x86_64-linux")]
    extra = [p for p in libs if os.path.isdir(p)]
    env["LD_LIBRARY_PATH"] = ":".join(extra + [env.get("LD_LIBRARY_PATH", "")])
    return env


def _compile(include_dir, main, tmp_path):
    import kwg

    if not shutil.which("g++"):
        pytest.skip("no g++")
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```cpp\n(.*?)```", text, re.S)
    assert len(blocks) >= 2
    src = tmp_path / "pricers.cpp"
    src.write_text("\n".join(blocks[:2]) + main)
    exe = tmp_path / "pricers"
    lib_dir = os.path.dirname(kwg.LIB_PATH)
    subprocess.run(["g++", "-std=c++20", "-I", include_dir, "-I", os.path.join(ROOT, "include"), str(src),
                    "-L", lib_dir, "-lkwg", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)], check=True)
    return str(exe)


def _init_only(exe):
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300, env=_env())
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() in ("init: []", "init: [Fd1dGpu_Pricer::init: no CUDA device]"), out.stdout


def test_integration_pricers_against_reference_headers(built, tmp_path):
    sys.path.insert(0, ROOT)
    import __graft_entry__ as ge

    if not os.path.isdir(ge.REF_SRC):
        pytest.skip("reference sources absent")
    _init_only(_compile(ge.REF_SRC, INIT_MAIN, tmp_path))


def test_integration_pricers_against_standin_headers(built, tmp_path):
    _init_only(_compile(STANDIN, INIT_MAIN, tmp_path))


def _price_through(exe, tmp_path, mode, opts, x_dim, t_dim, scale, density):
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    fin.write_bytes(np.ascontiguousarray(opts).tobytes())
    out = subprocess.run([exe, mode, str(x_dim), str(t_dim), repr(float(scale)), repr(float(density)), str(fin),
                          str(fout)], capture_output=True, text=True, timeout=600, env=_env())
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip() == f"price: [] {len(opts)}", out.stdout
    return np.fromfile(fout, dtype=np.float64)


def _rel(got, want, floor=PRICE_FLOOR):
    return float(np.max(np.abs(got - want) / np.maximum(np.abs(want), floor)))


@pytest.mark.gpu
def test_integration_pricers_price_on_the_gpu(built, tmp_path):
    import kwor

    exe = _compile(STANDIN, PRICE_MAIN, tmp_path)
    g = golden("pricer_test.npz")
    # the reference test's defaults: 512 x 512, scale 50, density 0.25
    p = _price_through(exe, tmp_path, "FD1D", g["opts"], 512, 512, 50.0, 0.25)
    assert _rel(p, g["ref_fd1d"]) <= REL_TOL
    assert np.max(np.abs(p - g["want"])) <= 1.3e-3  # test/kwPricer_test.cpp tolerance
    pbs = _price_through(exe, tmp_path, "FD1D-BS", g["opts"], 512, 512, 50.0, 0.25)
    assert _rel(pbs, g["ref_fd1d_bs"], BS_PRICE_FLOOR) <= REL_TOL
    q = golden("portfolio_qdfp.npz")
    p = _price_through(exe, tmp_path, "FD1D", q["opts"], 512, 512, 50.0, 0.25)
    assert _rel(p, q["ref_fd1d"]) <= REL_TOL
    assert np.max(np.abs(p - q["quantlib"])) <= 0.005  # test/kwPortfolio_test.cpp tolerance
    pbs = _price_through(exe, tmp_path, "FD1D-BS", q["opts"], 512, 512, 50.0, 0.25)
    rc, msg, want, _ = kwor.fd1d_price(q["opts"], bs=True, t_dim=512, x_dim=512, scale=50.0, density=0.25)
    assert rc == 0, msg
    assert _rel(pbs, want, BS_PRICE_FLOOR) <= REL_TOL

"""Host code under AddressSanitizer and UndefinedBehaviorSanitizer (CPU only).

* The library's parsers of untrusted input -- FLINT's table files (Tecplot
  ASCII and SZL binary, flint_files.cu) and the mechanism IR blob
  (flint_ir.cu) -- are compiled with -fsanitize=address,undefined together
  with tests/sanitize_host_parsers.cu and run on well-formed inputs and on
  truncated and byte-corrupted copies of them (seeded).  Every input must come
  back with a return code, and the sanitizers must report nothing.
* The FP64 oracle (oracle/flint_oracle.c) is compiled the same way and a child
  Python process (the sanitizer runtimes preloaded) runs the oracle's own
  tests against that build: source terms, Jacobians, the reactor, the general
  loop, cons2prim and transport.
"""
import os
import re
import shutil
import subprocess
import sys

import numpy as np
import pytest

from flint_gb300 import mechgen, tables
from flint_gb300.mech import Mechanism

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(REPO, "tests", "golden")
NVCC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
# one flag per entry: nvcc splits an -Xcompiler value at commas
SAN = ["-fsanitize=address", "-fsanitize=undefined", "-fno-omit-frame-pointer", "-fno-sanitize-recover=undefined"]
ENV_SAN = {"ASAN_OPTIONS": "detect_leaks=0:abort_on_error=0:halt_on_error=1",
           "UBSAN_OPTIONS": "print_stacktrace=1:halt_on_error=1"}
REPORT = re.compile(r"AddressSanitizer|runtime error:|UndefinedBehaviorSanitizer")


def _runtime(name):
    p = subprocess.run(["gcc", f"-print-file-name={name}"], capture_output=True, text=True).stdout.strip()
    return p if os.path.isabs(p) and os.path.exists(p) else None


def _build_parsers(out):
    if not os.path.exists(NVCC):
        pytest.skip("nvcc not found")
    csrc = os.path.join(REPO, "flint_gb300", "csrc")
    objs = []
    for src in (os.path.join(csrc, "flint_files.cu"), os.path.join(csrc, "flint_ir.cu"),
                os.path.join(REPO, "tests", "sanitize_host_parsers.cu")):
        obj = os.path.join(out, os.path.basename(src) + ".o")
        cmd = [NVCC, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O1", "-g", "-c", src, "-o", obj]
        for f in SAN:
            cmd += ["-Xcompiler", f]
        subprocess.run(cmd, check=True, capture_output=True)
        objs.append(obj)
    exe = os.path.join(out, "sanitize_host_parsers")
    cudalib = os.path.join(os.path.dirname(os.path.dirname(NVCC)), "lib64")
    subprocess.run(["g++", *SAN, "-o", exe, *objs, f"-L{cudalib}", "-lcudart", f"-Wl,-rpath,{cudalib}"],
                   check=True, capture_output=True)
    return exe


def _table_folders(root):
    """Well-formed ASCII and SZL table folders, then corrupted SZL copies."""
    mech = mechgen.load("c2")
    good = os.path.join(root, "ascii")
    tables.write_folder(tables.generate(mech, 300, 700), good)
    szl = os.path.join(root, "szl")
    shutil.copytree(good, szl)
    for base in ("thermo", "chemistry-Arrhenius", "chemistry-Troe", "chemistry-Lindemann"):
        p = os.path.join(szl, base + ".dat")
        if not os.path.exists(p):
            continue
        zones = tables.read_tecplot_points(p)
        with open(p) as f:
            names = re.findall(r'"([^"]*)"', [ln for ln in f if ln.startswith("VARIABLES")][0])
        tables.write_szplt(os.path.join(szl, base + ".szplt"), base, names, zones)
        os.remove(p)
    folders = [good, szl]
    rng = np.random.default_rng(11)
    blob = open(os.path.join(szl, "chemistry-Arrhenius.szplt"), "rb").read()
    cuts = sorted(set(int(c) for c in rng.integers(1, len(blob), 12))) + [8, 48, 64, 200]
    variants = [blob[:c] for c in cuts]
    for _ in range(24):   # byte flips, most of them in the header and tag tables
        b = bytearray(blob)
        for pos in rng.integers(0, min(len(b), 4096), 4):
            b[pos] = int(rng.integers(0, 256))
        variants.append(bytes(b))
    for i, v in enumerate(variants):
        d = os.path.join(root, f"bad{i}")
        shutil.copytree(szl, d)
        with open(os.path.join(d, "chemistry-Arrhenius.szplt"), "wb") as f:
            f.write(v)
        folders.append(d)
    trunc_dat = os.path.join(root, "bad_ascii")
    shutil.copytree(good, trunc_dat)
    p = os.path.join(trunc_dat, "thermo.dat")
    text = open(p).read()
    with open(p, "w") as f:
        f.write(text[: len(text) // 3])
    folders.append(trunc_dat)
    folders.append(os.path.join(root, "missing"))
    return folders


def _ir_blobs(root):
    rng = np.random.default_rng(12)
    paths = []
    for name in ("mech_pelucchi.json", "mech_wd.json", "mech_troyes.json"):
        blob = Mechanism.load(os.path.join(GOLD, name)).to_ir()
        variants = [blob, blob[: len(blob) // 2], blob[:16], b""]
        for _ in range(8):
            b = bytearray(blob)
            for pos in rng.integers(0, min(len(b), 256), 3):
                b[pos] = int(rng.integers(0, 256))
            variants.append(bytes(b))
        for i, v in enumerate(variants):
            p = os.path.join(root, f"{name}.{i}.ir")
            with open(p, "wb") as f:
                f.write(v)
            paths.append(p)
    return paths


def test_host_parsers_under_sanitizers(tmp_path):
    if _runtime("libasan.so") is None:
        pytest.skip("no AddressSanitizer runtime")
    exe = _build_parsers(str(tmp_path))
    args = []
    for d in _table_folders(str(tmp_path / "tables")):
        args += ["--tables", d, ""]
    for p in _ir_blobs(str(tmp_path)):
        args += ["--ir", p]
    r = subprocess.run([exe, *args], capture_output=True, text=True, env={**os.environ, **ENV_SAN}, timeout=600)
    out = r.stdout + r.stderr
    assert r.returncode == 0 and not REPORT.search(out), out[-4000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith(("tables", "ir "))]
    assert len(lines) == len([a for a in args if a in ("--tables", "--ir")])
    assert " rc=0 " in lines[0] and " rc=0 " in lines[1]             # the well-formed ASCII and SZL folders
    assert any(ln.startswith("ir ") and " rc=0 " in ln for ln in lines)
    assert any(" rc=0 " not in ln for ln in lines)                    # the corrupted inputs are refused


def test_oracle_under_sanitizers(tmp_path):
    asan, ubsan = _runtime("libasan.so"), _runtime("libubsan.so")
    if asan is None or ubsan is None:
        pytest.skip("no sanitizer runtimes")
    so = str(tmp_path / "liboracle_san.so")
    src = os.path.join(REPO, "oracle", "flint_oracle.c")
    subprocess.run(["gcc", "-O1", "-g", "-fPIC", "-std=c11", "-ffp-contract=off", "-fopenmp", *SAN, "-shared",
                    "-o", so, src, "-lm"], check=True, capture_output=True)
    env = {**os.environ, **ENV_SAN, "LD_PRELOAD": f"{asan}:{ubsan}", "FLINT_ORACLE_SO": so, "OMP_NUM_THREADS": "2"}
    probe = subprocess.run([sys.executable, "-c", "from oracle.oracle import lib; print(lib()._name)"],
                           capture_output=True, text=True, env=env, cwd=REPO, timeout=300)
    assert probe.stdout.strip() == so, probe.stdout + probe.stderr    # the sanitized build is the one loaded
    tests = [os.path.join(REPO, "tests", t) for t in
             ("test_oracle_golden.py", "test_oracle_jacobian.py", "test_oracle_reactor.py", "test_cons2prim.py",
              "test_transport.py")]
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-p", "no:cacheprovider", "-m", "not gpu",
                        *tests], capture_output=True, text=True, env=env, cwd=REPO, timeout=1200)
    out = r.stdout + r.stderr
    assert r.returncode == 0 and not REPORT.search(out), out[-4000:]

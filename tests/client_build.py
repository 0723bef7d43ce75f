"""Compile tests/client/hepem_client.cpp, a C++ client of the library that
uses include/g4hepem_gb300.hh as a G4HepEm client would, against the built
libg4hepem_gb300.so (g++ and the CUDA runtime, no CMake)."""
from __future__ import annotations

import os
import subprocess

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(REPO, "tests", "client", "hepem_client.cpp")
OUT_DIR = os.path.join(REPO, "tests", "client", "_build")
OUT = os.path.join(OUT_DIR, "hepem_client")
LIBDIR = os.path.join(REPO, "g4hepem_gb300")


def cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.isdir(os.path.join(c, "include")):
            return c
    raise RuntimeError("CUDA toolkit not found")


def build_client() -> str:
    from g4hepem_gb300 import build as B
    B.build()
    deps = [SRC, os.path.join(REPO, "include", "g4hepem_gb300.hh"), os.path.join(REPO, "include", "g4hepem_gb300.h"),
            B.OUT]
    if os.path.exists(OUT) and all(os.path.getmtime(d) <= os.path.getmtime(OUT) for d in deps):
        return OUT
    os.makedirs(OUT_DIR, exist_ok=True)
    cuda = cuda_home()
    lib64 = os.path.join(cuda, "lib64")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", os.path.join(REPO, "include"), "-I",
           os.path.join(cuda, "include"), SRC, "-o", OUT, "-L", LIBDIR, "-lg4hepem_gb300", f"-Wl,-rpath,{LIBDIR}",
           "-L", lib64, "-lcudart", f"-Wl,-rpath,{lib64}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"client build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return OUT


TRACE_SRC = os.path.join(REPO, "tests", "trace", "trace_recorder.c")
TRACE_OUT = os.path.join(REPO, "tests", "trace", "_build", "trace_recorder.so")


def build_trace_recorder() -> str:
    """Compile tests/trace/trace_recorder.c, the NVTX injection library that
    records the library's ranges (gcc and the NVTX headers of the toolkit)."""
    if os.path.exists(TRACE_OUT) and os.path.getmtime(TRACE_SRC) <= os.path.getmtime(TRACE_OUT):
        return TRACE_OUT
    os.makedirs(os.path.dirname(TRACE_OUT), exist_ok=True)
    cmd = ["gcc", "-std=c99", "-O2", "-Wall", "-Wextra", "-fPIC", "-shared", "-I",
           os.path.join(cuda_home(), "include"), TRACE_SRC, "-o", TRACE_OUT]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"trace recorder build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return TRACE_OUT


def run_traced(code: str, log_path: str, timeout: float = 600) -> list:
    """Run `code` in a fresh python process with the trace recorder injected;
    returns the recorded lines split into fields."""
    import sys
    env = dict(os.environ)
    env["NVTX_INJECTION64_PATH"] = build_trace_recorder()
    env["HEPEM_TRACE_LOG"] = log_path
    env["PYTHONPATH"] = os.pathsep.join([REPO, os.path.join(REPO, "tests"), env.get("PYTHONPATH", "")])
    r = subprocess.run([sys.executable, "-c", code], env=env, cwd=REPO, capture_output=True, text=True,
                       timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"traced run failed:\n{r.stdout}\n{r.stderr}")
    with open(log_path) as f:
        return [line.split() for line in f if line.strip()]

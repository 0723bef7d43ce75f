"""The C++ client (tests/client/hepem_client.cpp) builds against
include/g4hepem_gb300.hh and the library, and runs what needs no GPU: the
table image of a JSON document and its check, a damaged image rejected, the
status strings, the step-limit record size; without a device, creating the
tables is a HEPEM_NO_DEVICE error, not a crash."""
import re
import subprocess

from client_build import build_client
from conftest import T3, T16


def test_cpp_client_builds_and_runs_without_gpu():
    exe = build_client()
    for table in (T3, T16):
        r = subprocess.run([exe, "info", table], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stderr
        out = r.stdout
        m = re.search(r"image_bytes (\d+) arena_bytes (\d+) damaged_image_status (\d+)", out)
        assert m and int(m.group(1)) > int(m.group(2)) > 100000
        assert int(m.group(3)) == 2  # HEPEM_PARSE_ERROR
        assert re.search(r"limit_bytes_1000 (\d+)", out).group(1) != "0"
        assert "status 0 ok" in out and "status 7 no CUDA device" in out
        assert ("no-device" in out) or re.search(r"device couples (\d+) \1", out)


def test_cpp_client_usage_error():
    exe = build_client()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "usage" in r.stderr
    r = subprocess.run([exe, "info", "/nonexistent/table.json"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "cannot read" in r.stderr

"""NVTX ranges of the library (domain "g4hepem_gb300"), recorded by the test
injection library tests/trace/trace_recorder.c, without a GPU: the table
image calls open and close one range each, with the document's or image's
size as payload; without an injection library the calls record nothing and
behave as before."""
import os

from client_build import run_traced
from conftest import T3

CODE = """
import ctypes as C
from g4hepem_gb300 import native
L = native.lib()
doc = open({table!r}, 'rb').read()
img = native.image_from_json(doc)
arena = C.c_int64(0)
assert L.hepem_image_check(img, len(img), C.byref(arena)) == 0
assert L.hepem_image_check(b'bad', 3, C.byref(arena)) != 0
print(len(doc), len(img))
"""


def test_image_calls_record_ranges(tmp_path):
    log = str(tmp_path / "trace.log")
    ev = run_traced(CODE.format(table=T3), log)
    doc_len, img_len = os.path.getsize(T3), None
    pushes = [e for e in ev if e[0] == "push"]
    pops = [e for e in ev if e[0] == "pop"]
    assert all(e[1] == "g4hepem_gb300" for e in ev), ev
    names = [e[2] for e in pushes]
    # two image_from_json calls (size query, then the copy), two checks
    assert names == ["hepem_image_from_json"] * 2 + ["hepem_image_check"] * 2, names
    assert int(pushes[0][3]) == doc_len and int(pushes[1][3]) == doc_len
    img_len = int(pushes[2][3])
    assert img_len > doc_len // 10 and int(pushes[3][3]) == 3
    # every range closed, in order (depth never negative, ends at 0)
    depth = 0
    for e in ev:
        depth += 1 if e[0] == "push" else -1
        assert depth >= 0
    assert depth == 0 and len(pops) == len(pushes)

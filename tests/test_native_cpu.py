"""CPU tests of the C-ABI library: it loads, exports every declared entry
point, and rejects malformed table documents on the host (the JSON is parsed
and validated before any device work, so these run without a GPU)."""
import json
import os
import re

import numpy as np
import pytest

from conftest import REPO, T3, has_gpu
from g4hepem_gb300 import workload as W


def declared_entry_points():
    text = open(os.path.join(REPO, "include", "g4hepem_gb300.h")).read()
    return sorted(set(re.findall(r"\b(hepem_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(native):
    L = native.lib()
    decl = declared_entry_points()
    assert len(decl) >= 10
    for name in decl:
        assert hasattr(L, name), name
    assert set(native.EXPORTED) <= set(decl)


def test_status_strings(native):
    L = native.lib()
    for code in range(9):
        assert len(L.hepem_status_string(code)) > 0


def test_philox_host_function_matches_stream_contract(native):
    ids = np.array([0, 5, 99999], dtype=np.int32)
    want = W.philox_uniforms(1234567, ids, 9)
    got = np.array([[native.philox_uniform(1234567, int(i), k) for k in range(9)] for i in ids])
    assert np.array_equal(want, got)


def _doc():
    return json.load(open(T3))


@pytest.mark.parametrize("mutate,needle", [
    (lambda d: d["fData"].pop("fTheGammaData"), "fTheGammaData"),
    (lambda d: d["fData"]["fTheMatCutData"]["fMatCutData"][1].__setitem__("fHepEmMatIndex", 7), "material index"),
    (lambda d: d["fData"]["fTheMatCutData"]["fMatCutData"][0].__setitem__("fG4RegionIndex", 3), "region index"),
    (lambda d: d["fData"]["fTheElectronData"]["fELossData"].pop(), "fELossData size"),
    (lambda d: d["fData"]["fTheElectronData"]["fResMacXSecStartIndexPerMatCut"].__setitem__(2, 10**7), "xs start"),
    (lambda d: d["fData"]["fTheSBTableData"]["fSBStartTablesStartPerZ"].__setitem__(82, 10**8), "SB start"),
    (lambda d: d["fData"]["fTheGammaData"].__setitem__("fDataPerMat", 7), "gamma table sizes"),
    (lambda d: d["fData"]["fTheMaterialData"]["fMaterialData"][0]["fElementVect"].__setitem__(0, 300), "Z out of"),
])
def test_malformed_state_is_a_parse_error(native, mutate, needle):
    d = _doc()
    mutate(d)
    with pytest.raises(native.HepEmError) as e:
        native.Context(json_text=json.dumps(d))
    assert e.value.code == 2
    assert needle in str(e.value), str(e.value)


def test_truncated_json_is_a_parse_error(native):
    text = open(T3).read()[:5000]
    with pytest.raises(native.HepEmError) as e:
        native.Context(json_text=text)
    assert e.value.code == 2


def test_missing_file(native):
    with pytest.raises(native.HepEmError) as e:
        native.Context(json_path="/nonexistent/state.json")
    assert e.value.code == 2


@pytest.mark.skipif(has_gpu(), reason="checks the no-device path")
def test_valid_state_without_device_reports_no_device(native):
    with pytest.raises(native.HepEmError) as e:
        native.Context(T3)
    assert e.value.code == 7


def test_arena_image_round_trip_and_damage(native):
    from conftest import T3, T16
    for path in (T3, T16):
        text = open(path, "rb").read()
        img = native.image_from_json(text)
        assert img[:8] == b"HEPEMIMG"
        assert img == native.image_from_json(text)           # deterministic
        nb = native.image_check(img)
        assert 0 < nb < len(img)
    # damaged images are parse errors, never accepted
    bad = bytearray(img)
    bad[len(bad) // 2] ^= 0x40
    for b in (bytes(bad), img[:-9], img[:100], b"HEPEMIMG" + b"\0" * 64):
        with pytest.raises(native.HepEmError) as e:
            native.image_check(b)
        assert e.value.code == 2
    with pytest.raises(native.HepEmError) as e:
        native.image_from_json(b'{"fParameters": {}}')
    assert e.value.code == 2


def test_context_from_image_without_device_reports_no_device(native):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from conftest import T3
    img = native.image_from_json(open(T3, "rb").read())
    with pytest.raises(native.HepEmError) as e:
        native.Context(image=img)
    assert e.value.code == 7

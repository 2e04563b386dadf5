"""CPU tests of the C ABI: the library loads, exports every symbol the header
declares, and fails cleanly (no crash, a status code) where no GPU is visible."""
import ctypes as C
import os
import re

import pytest

from conftest import ROOT


def _header_functions():
    with open(os.path.join(ROOT, "include", "ohpic.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ohpic_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_the_path():
    names = _header_functions()
    for must in ("ohpic_create", "ohpic_scatter", "ohpic_solve", "ohpic_interp", "ohpic_move",
                 "ohpic_push", "ohpic_step", "ohpic_sort", "ohpic_upload_particles",
                 "ohpic_download_particles", "ohpic_diagnostics", "ohpic_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(ohpic):
    L = C.CDLL(ohpic.LIB_PATH)
    names = _header_functions()
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # the Python binding covers exactly the declared functions
    assert sorted(ohpic.SIGNATURES) == names


def test_config_default(ohpic):
    cfg = ohpic.default_config()
    assert cfg.precision == ohpic.FP64
    assert cfg.weights == ohpic.WEIGHTS_REFERENCE
    assert cfg.sort_every == 20 and cfg.track_ids == 1 and cfg.device == 0
    assert cfg.nx == 0 and cfg.nspecies == 0


def test_status_strings(ohpic):
    L = ohpic.lib()
    for code in range(0, 10):
        assert L.ohpic_status_string(code)
    assert L.ohpic_status_string(ohpic.ERR_UNSUPPORTED).decode().startswith("per-particle")


def test_invalid_configs_rejected_before_device(ohpic):
    """Argument checks run before any CUDA call, so they hold on any host."""
    base = dict(n=(8, 8, 8), dt=0.1, b0=(0, 0, 0), qm=[-1.0], q=[-0.1], capacity=[16])
    bad = [
        dict(base, n=(0, 8, 8)),
        dict(base, qm=[0.0]),
        dict(base, capacity=[-1]),
        dict(base, n=(12, 8, 8), tile=(8, 8, 8)),       # tile must divide n
        dict(base, n=(4096, 8, 8), precision=1),         # FP32 cell packing limit
    ]
    for kw in bad:
        cfg = ohpic.make_config(**kw)
        with pytest.raises(ohpic.OhpicError) as e:
            ohpic.PicContext(cfg)
        assert e.value.status == ohpic.ERR_INVALID
    cfg = ohpic.make_config(**base)
    cfg.nspecies = 9
    with pytest.raises(ohpic.OhpicError):
        ohpic.PicContext(cfg)


def test_null_arguments(ohpic):
    L = ohpic.lib()
    assert L.ohpic_create(None, None) == ohpic.ERR_INVALID
    assert L.ohpic_destroy(None) == ohpic.OK
    assert L.ohpic_scatter(None) == ohpic.ERR_INVALID
    assert L.ohpic_step(None, 0.1, 1) == ohpic.ERR_INVALID

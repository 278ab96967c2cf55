import glob
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 and the CUDA build")


def golden_names():
    return sorted(os.path.splitext(os.path.basename(p))[0]
                  for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def golden_index():
    with open(os.path.join(GOLDEN, "index.json"), encoding="utf-8") as f:
        return json.load(f)


def cfg_from(arr, mod):
    a = [int(v) for v in arr]
    return mod.GrandDecoderConfig(*a) if hasattr(mod, "GrandDecoderConfig") else mod.Config(*a)


@pytest.fixture(scope="session")
def port():
    import oracle as O
    O.build()
    return O.Port()


@pytest.fixture(scope="session")
def gpulib():
    """The CUDA library, built in-tree; a GPU test fails loudly without it."""
    from library_s_grand_gb300 import build as B
    from library_s_grand_gb300 import capi
    B.build()
    return capi.load_library()


def write_aux(tmp_path, g):
    """Re-create the phase-mask / LLR file a golden fixture was decoded with."""
    if "phase_text" in g:
        p = tmp_path / "phase.txt"
        p.write_text(str(g["phase_text"]))
        return str(p)
    if "file_text" in g:
        p = tmp_path / "aux.txt"
        p.write_text(str(g["file_text"]))
        return str(p)
    return None

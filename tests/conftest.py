import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HERE = os.path.dirname(os.path.abspath(__file__))
for p in (HERE, os.path.join(ROOT, "micsa-ea-mc_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")
    config.addinivalue_line("markers", "reference: needs the reference sources (CPU build of it)")


def _ensure_built():
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "micsa_build", os.path.join(ROOT, "micsa-ea-mc_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()
    import oracle
    oracle.build()


_ensure_built()


def golden_cases(max_volume=None):
    import glob
    import json
    out = []
    for f in sorted(glob.glob(os.path.join(HERE, "golden", "*.json"))):
        g = json.load(open(f))
        if max_volume is None or g["cfg"]["L"] ** 3 * g["cfg"]["nr"] <= max_volume:
            out.append(pytest.param(g, id=os.path.basename(f)[:-5]))
    return out


def cuda_device_count():
    try:
        import torch
        return torch.cuda.device_count() if torch.cuda.is_available() else 0
    except Exception:
        return 0

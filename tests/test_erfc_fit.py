"""The FP32 Ewald screening function of the pair kernels (erfc_scaled in
sdm_kernels.cu): its constants, read from the CUDA source, evaluated the way
the kernel does (FP32 Horner, FP32 exponential), against scipy's erfc."""
import os
import re

import numpy as np
import pytest

scipy_special = pytest.importorskip("scipy.special")

SRC = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "openmm_sdm_plugin_gb300", "csrc",
                   "sdm_kernels.cu")


def _constants():
    s = open(SRC).read()
    p = float(re.search(r"kErfcP = ([0-9.eE+-]+)f;", s).group(1))
    body = re.search(r"float erfc_scaled\(float x\) \{(.*?)\n\}", s, re.S).group(1)
    nums = [float(v) for v in re.findall(r"(-?[0-9]+\.[0-9]+(?:[eE][+-]?[0-9]+)?)f", body)]
    # t = 1 / (1 + p x), then Horner from c7 down to c0
    assert nums[0] == 1.0
    return p, nums[1:][::-1]


def test_screening_constants_and_error():
    import sys
    sys.path.insert(0, os.path.dirname(SRC))
    try:
        import fit_erfc
    finally:
        sys.path.pop(0)
    p, c = _constants()
    assert len(c) == 8
    x = np.linspace(0.0, 4.0, 200001)
    v = fit_erfc.eval_f32(c, p, x)
    ref = scipy_special.erfc(x.astype(np.float32).astype(np.float64))
    assert np.abs(v / ref - 1.0).max() < 6e-7
    # the kernel's source holds the packed and the scalar form with the same numbers
    s = open(SRC).read()
    packed = re.search(r"float2 erfc_scaled2\(float2 x\) \{(.*?)\n\}", s, re.S).group(1)
    for ck in c:
        assert repr(ck) in packed or f"{ck}" in packed

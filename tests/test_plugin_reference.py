"""The reference-side box class (tensorsat_gb300.plugin) obeys the upstream metaclass
rules. Runs only where the upstream sources are available (fixture containers); skipped
elsewhere."""

from __future__ import annotations

import sys
from pathlib import Path

import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def _upstream():
    sys.path.insert(0, str(GOLDEN))
    import _ref_import

    if not _ref_import.available():
        pytest.skip("upstream tensorsat sources not available")
    _ref_import.install()
    import tensorsat

    return tensorsat


def test_finrel_cuda_is_a_final_contractible_upstream_box():
    tensorsat = _upstream()
    import torch

    from tensorsat_gb300.plugin import make_finrel_cuda

    cls = make_finrel_cuda(tensorsat)
    from tensorsat.diagrams import Box, TensorLikeBox

    assert issubclass(cls, TensorLikeBox)
    assert cls.__final__ and cls.can_be_contracted()
    box = cls._new(torch.zeros(2, 3, dtype=torch.uint8))
    assert box.tensor_shape == (2, 3)
    assert Box.class_join([cls, cls]) is cls

"""The device-adapter tag's C++ test program (tests/tag/test_tag.cpp) builds:
include/dax_gb300_tag.h compiles against the DaxToolkit's own control
headers (or, without the reference tree, the exported preprocessed copy
does) and links the C ABI.  It runs under -m gpu (tests/test_tag_gpu.py)."""
import os

import pytest


def test_tag_program_builds():
    from tests.tag import build
    path = build.build()
    if path is None:
        pytest.skip("neither the DaxToolkit tree nor an exported test_tag source is present")
    assert os.path.exists(path) and os.access(path, os.X_OK)

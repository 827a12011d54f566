"""The reference's GPU kernels compile from their sources for sm_103a (the
second oracle of tests/test_gpu_ref_kernels.py); only where the reference
tree is present."""
import pytest

from oracle import build_oracle as O


def test_reference_kernels_compile():
    if not (O.REF_ROOT / "Born").is_dir():
        pytest.skip("the reference tree is not present")
    path = O.build_ref_kernels()
    assert path is not None and path.exists() and path.stat().st_size > 0

"""Host volumes through the library's copies: a dense host volume goes to the
pitched device layout and back bit for bit (flat copies through the staging
buffer, re-pitched on the device by a kernel), for a row length that allows
16-byte accesses and for one that does not, and for volumes larger than one
staging chunk."""
import numpy as np
import pytest

from sep_code_gb300 import gpu_funcs as gf

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [(17, 20, 18), (96, 80, 64), (560, 560, 80)])
def test_volume_round_trip(n):
    n1, n2, n3 = n
    gf.setup_cuda(1)
    gf.create_gpu_space(10.0, 10.0, 10.0, 20.0, 0.002, 0.002, n1, n2, n3)
    rng = np.random.default_rng(n1)
    vol = rng.standard_normal((n3, n2, n1)).astype(np.float32)
    gf.set_image(vol)
    back = gf.get_image((n3, n2, n1))
    assert np.array_equal(back, vol)
    # twice in a row: the staging buffer is reused
    vol2 = -vol
    gf.set_image(vol2)
    assert np.array_equal(gf.get_image((n3, n2, n1)), vol2)

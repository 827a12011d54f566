"""SEP datasets straight to and from device vectors (include/sepx_sepio.h,
on_device = 1): pinned staging buffers, the big-endian byte swap on the GPU.
A 48 MB dataset (larger than one 32 MB staging buffer, so both buffers
alternate) and a window of it, bit for bit against numpy's own reading of
the same files."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.mark.parametrize("xdr", [True, False])
def test_device_read_write_bit_exact(tmp_path, xdr):
    from sep_code_gb300 import gpu_funcs as gf
    from sep_code_gb300 import sepio as S
    gf.setup_cuda(1)
    rng = np.random.default_rng(6)
    a = rng.standard_normal((12, 1000, 1000)).astype(np.float32)
    p = tmp_path / "big.H"
    S.write(p, a, o=[0.0, 0.0, 0.0], d=[0.004, 12.5, 12.5], xdr=xdr)
    dev = torch.empty(a.size, device="cuda")
    torch.cuda.synchronize()
    S.read_to_device(p, dev.data_ptr())
    assert np.array_equal(dev.cpu().numpy().view(np.uint32), a.ravel().view(np.uint32))
    q = tmp_path / "back.H"
    S.write_from_device(q, dev.data_ptr(), [1000, 1000, 12], d=[0.004, 12.5, 12.5], xdr=xdr)
    raw = np.fromfile(str(q) + "@", ">f4" if xdr else "<f4").astype(np.float32)
    assert np.array_equal(raw.view(np.uint32), a.ravel().view(np.uint32))
    # part of the data, from an element offset
    part = torch.zeros(12345, device="cuda")
    torch.cuda.synchronize()
    S.read_to_device(p, part.data_ptr(), first=777, count=12345)
    assert np.array_equal(part.cpu().numpy(), a.ravel()[777:777 + 12345])
    # a strided window
    win = torch.zeros(300 * 250 * 5, device="cuda")
    torch.cuda.synchronize()
    S.read_window_to_device(p, win.data_ptr(), [300, 250, 5], [7, 11, 2], [3, 2, 2])
    want = a[2:11:2, 11:11 + 2 * 249 + 1:2, 7:7 + 3 * 299 + 1:3]
    assert np.array_equal(win.cpu().numpy().reshape(want.shape), want)

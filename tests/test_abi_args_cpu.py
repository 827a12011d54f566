"""Argument checks of the C ABI entry points, on the CPU: a NULL host or
device buffer, a negative length or an oversized receiver grid is an error
with a message, checked before any device state is touched (so no GPU is
needed here), instead of a host crash or a kernel reading address 0."""
import ctypes as C

import numpy as np
import pytest

VP = C.c_void_p


@pytest.fixture(scope="module")
def raw():
    """The library with untyped pointer arguments, so that NULL can be passed."""
    from sep_code_gb300 import build
    from sep_code_gb300._lib import lib  # noqa: F401  (builds the library if needed)
    L = C.CDLL(str(build.LIB))
    L.sepx_last_error.restype = C.c_char_p
    return L


def _rejects(L, rc, word):
    assert rc != 0
    msg = L.sepx_last_error()
    assert word.encode() in msg, msg


def test_reference_named_calls_reject_null_buffers(raw):
    L = raw
    f = np.zeros(64, np.float32)
    i = np.zeros(64, np.int32)
    fp, ip = VP(f.ctypes.data), VP(i.ctypes.data)
    _rejects(L, L.sepx_transfer_vel_func1(4, 4, 4, None), "NULL")
    _rejects(L, L.sepx_transfer_source_func(9, 10, None, fp), "NULL")
    _rejects(L, L.sepx_transfer_source_func(9, 10, ip, None), "NULL")
    _rejects(L, L.sepx_transfer_source_func(-1, 10, ip, fp), "invalid source shape")
    _rejects(L, L.sepx_transfer_receiver_func(2, 2, 10, None, fp), "NULL")
    _rejects(L, L.sepx_transfer_receiver_func(2, 2, 10, ip, None), "NULL")
    _rejects(L, L.sepx_transfer_receiver_func(70000, 70000, 10, ip, fp), "too many receivers")
    _rejects(L, L.sepx_set_receivers(2, 2, 10, None), "NULL")
    _rejects(L, L.sepx_source_prop(4, 4, 4, C.c_bool(False), C.c_bool(True), None, fp, 1, 9, 10),
             "NULL")
    _rejects(L, L.sepx_rtm_forward(4, 4, 4, 1, None, fp, 9, 10, 18, 2, 2), "NULL")
    _rejects(L, L.sepx_rtm_forward(4, 4, 4, 1, fp, None, 9, 10, 18, 2, 2), "NULL")
    _rejects(L, L.sepx_rtm_adjoint(4, 4, 4, 1, None, fp, fp, 9, 10), "NULL")
    _rejects(L, L.sepx_rtm_adjoint(4, 4, 4, 1, fp, fp, None, 9, 10), "NULL")
    _rejects(L, L.sepx_set_image(None), "NULL")
    _rejects(L, L.sepx_get_image(None), "NULL")
    _rejects(L, L.sepx_set_source_fields(fp, None), "NULL")
    _rejects(L, L.sepx_get_source_fields(None, fp), "NULL")


def test_device_vector_calls_reject_null_and_negative_lengths(raw):
    L = raw
    f = np.zeros(64, np.float32)
    fp = VP(f.ctypes.data)
    n = C.c_longlong
    out = C.c_double()
    _rejects(L, L.sepx_vec_alloc(None, n(10)), "NULL")
    _rejects(L, L.sepx_vec_upload(None, fp, n(10)), "NULL")
    _rejects(L, L.sepx_vec_download(fp, None, n(10)), "NULL")
    _rejects(L, L.sepx_vec_fill(fp, n(-1), C.c_float(0.0)), "negative length")
    _rejects(L, L.sepx_vec_scale_add2(fp, fp, None, n(8), C.c_double(1), C.c_double(1)), "NULL")
    _rejects(L, L.sepx_vec_random(None, n(8), C.c_ulonglong(1)), "NULL")
    _rejects(L, L.sepx_dot_f32(None, None, n(5), C.byref(out)), "NULL")
    _rejects(L, L.sepx_dot_f32(fp, None, n(5), None), "NULL")
    _rejects(L, L.sepx_op_image_to_padded(None, 4, 4, 4, 0, 0, 0), "NULL")
    _rejects(L, L.sepx_op_traces_to_data(None, 10, C.c_float(0.001)), "NULL")


def test_unet_calls_reject_null_operands(raw):
    """A NULL device operand of the U-Net kernels is an error, not a launch
    that reads address 0; an empty element-wise call is a no-op."""
    L = raw
    p = VP(16)   # never dereferenced: every call below fails or returns first
    n = C.c_longlong
    _rejects(L, L.sepx_unet_pack_weights(None, 8, 8, 27, 0, p, None), "NULL")
    _rejects(L, L.sepx_unet_conv_fwd(None, 8, 0, 1, 4, 8, 8, 8, 27, p, None, 8, 0, p, 8, 0,
                                     None, None, None), "NULL")
    _rejects(L, L.sepx_unet_conv_fwd(p, 8, 0, 1, 4, 8, 8, 8, 27, None, None, 8, 0, p, 8, 0,
                                     None, None, None), "NULL")
    _rejects(L, L.sepx_unet_conv_fwd(p, 8, 0, 1, 4, 8, 8, 8, 27, p, None, 8, 0, None, 8, 0,
                                     None, None, None), "no output")
    _rejects(L, L.sepx_unet_conv_fwd(p, 8, 0, 0, 4, 8, 8, 8, 27, p, None, 8, 0, p, 8, 0,
                                     None, None, None), "empty volume")
    _rejects(L, L.sepx_unet_conv_wgrad(p, 8, 0, 1, 4, 8, 8, 8, 27, None, 8, 0, 8, p, None), "NULL")
    _rejects(L, L.sepx_unet_avgpool(p, 8, 0, 1, 4, 8, 8, 8, None, 8, 0, None), "NULL")
    _rejects(L, L.sepx_unet_upsample_bwd(None, 8, 0, 1, 4, 8, 8, 8, p, 8, 0, None), "NULL")
    _rejects(L, L.sepx_unet_adam(p, None, p, p, n(8), C.c_float(1e-3), C.c_float(0.9),
                                 C.c_float(0.999), C.c_float(1e-8), 1, None), "NULL")
    _rejects(L, L.sepx_unet_conv_wgrad_bias(p, 8, 0, 1, 4, 8, 8, 8, 27, None, 8, 0, 8, p, p, None),
             "NULL")
    _rejects(L, L.sepx_unet_conv_wgrad_bias(p, 8, 0, 1, 4, 8, 8, 8, 27, p, 8, 0, 8, None, p, None),
             "NULL")
    _rejects(L, L.sepx_unet_bias_grad(p, 12, 0, n(4), 8, p, None), "bad channel")
    _rejects(L, L.sepx_unet_adam_dev(p, p, p, p, n(8), None, None), "NULL")
    assert L.sepx_unet_set_wgrad_form(3) == -1
    _rejects(L, L.sepx_unet_pack_weights_many(65, p, p, p, p, p, p, None), "jobs")
    _rejects(L, L.sepx_unet_pack_weights_many(2, None, p, p, p, p, p, None), "NULL")
    assert L.sepx_unet_pack_weights_many(0, None, None, None, None, None, None, None) == 0
    _rejects(L, L.sepx_unet_adam_dev(p, p, p, p, n(-1), p, None), "n -1")
    assert L.sepx_unet_adam_dev(None, None, None, None, n(0), None, None) == 0
    _rejects(L, L.sepx_unet_capture_begin(None), "legacy stream")
    _rejects(L, L.sepx_unet_capture_end(None, None), "NULL")
    _rejects(L, L.sepx_unet_graph_launch(None, None), "NULL handle")
    assert L.sepx_unet_graph_free(None) == 0
    _rejects(L, L.sepx_unet_mse(p, p, n(-1), p, 8, p, None), "negative length")
    assert L.sepx_unet_to_bf16(None, n(0), C.c_float(1.0), None, 8, 0, None) == 0

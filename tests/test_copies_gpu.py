"""lne_copy_to_host / lne_copy_to_device through the C ABI: page-locked,
mapped host buffers go through the SM copy kernel (including sizes and
offsets off the 16-byte grid), pageable ones through cudaMemcpyAsync; the
bytes must arrive unchanged either way."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nbytes,offset", [(16 << 20, 0), ((3 << 20) + 7, 3), ((2 << 20) + 9, 16), (1000, 1)])
@pytest.mark.parametrize("pinned", [True, False])
def test_copy_round_trip(ctx, lib, nbytes, offset, pinned):
    rng = np.random.default_rng(nbytes + offset)
    src = torch.from_numpy(rng.integers(0, 256, nbytes + 64, dtype=np.uint8))
    back = torch.zeros(nbytes + 64, dtype=torch.uint8)
    if pinned:
        src, back = src.pin_memory(), back.pin_memory()
    dev = torch.zeros(nbytes + 64, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    rc = lib.lne_copy_to_device(ctx.handle, ctypes.c_void_p(dev.data_ptr() + offset),
                                ctypes.c_void_p(src.data_ptr() + offset), nbytes)
    assert rc == 0, lib.lne_last_error()
    d = dev.cpu().numpy()
    assert np.array_equal(d[offset:offset + nbytes], src.numpy()[offset:offset + nbytes])
    assert not d[:offset].any() and not d[offset + nbytes:].any()
    rc = lib.lne_copy_to_host(ctx.handle, ctypes.c_void_p(back.data_ptr() + offset),
                              ctypes.c_void_p(dev.data_ptr() + offset), nbytes)
    assert rc == 0, lib.lne_last_error()
    b = back.numpy()
    assert np.array_equal(b[offset:offset + nbytes], src.numpy()[offset:offset + nbytes])
    assert not b[:offset].any() and not b[offset + nbytes:].any()

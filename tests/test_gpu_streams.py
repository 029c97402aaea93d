"""GPU: a handle leaves a caller's CUDA stream as it found it.

dfpt_set_stream lets the caller's stream carry the handle's work. The handle's L2 residency window
over its traversal records belongs on its own graphs' kernel nodes, never on a stream that outlives
the handle: after rendering and after dfpt_destroy, the caller's stream has no access-policy window
(read back through the driver API's cuStreamGetAttribute).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CU_STREAM_ATTRIBUTE_ACCESS_POLICY_WINDOW = 1


def _window_bytes(cuda_stream):
    cuda = C.CDLL("libcuda.so.1")
    cuda.cuStreamGetAttribute.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    cuda.cuStreamGetAttribute.restype = C.c_int
    value = (C.c_uint8 * 64)()  # CUstreamAttrValue; accessPolicyWindow = {base_ptr, num_bytes, ...}
    rc = cuda.cuStreamGetAttribute(C.c_void_p(cuda_stream), CU_STREAM_ATTRIBUTE_ACCESS_POLICY_WINDOW, value)
    assert rc == 0, rc
    return int(np.frombuffer(bytes(value), np.uint64)[1])


def test_caller_stream_keeps_no_l2_window():
    import torch
    from dfpt import synthetic
    from dfpt.kernel import RendererKernel

    scene, sky, params, (w, h) = synthetic.small_mesh_scene(width=64, height=48)
    stream = torch.cuda.Stream()
    assert _window_bytes(stream.cuda_stream) == 0
    k = RendererKernel(scene, sky, params)
    k.update(w, h)
    k.set_tuning("l2_persist", 1)
    k.set_stream(stream.cuda_stream)
    k.execute(3)
    k.synchronize()
    film, n = k.film()
    assert (n == 3).all() and np.isfinite(film).all()
    assert _window_bytes(stream.cuda_stream) == 0
    k.dispose()
    assert _window_bytes(stream.cuda_stream) == 0
    # The stream still works for other work after the handle is gone.
    with torch.cuda.stream(stream):
        x = torch.ones(1024, device="cuda") * 2
    stream.synchronize()
    assert float(x.sum()) == 2048.0

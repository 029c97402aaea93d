"""dfpt_film_mean_noalloc, the allocation-free image-mean entry point (collected last).

Callers that cannot allocate device memory while they run (a frame loop that must not call
cudaMalloc/cudaFree, a host whose device memory belongs to another allocator) pass the film and
the output in device memory; the reduction's scratch is a fixed device array inside the library.
This test calls it through the C-ABI twice in a row and checks each result against the
allocating entry point, dfpt_read_film_mean, to a relative 1e-9 (both reduce the same float film
in FP64, in different orders).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_film_mean_noalloc_matches_read_film_mean():
    import torch

    from dfpt import _lib, synthetic
    from dfpt.kernel import RendererKernel

    lib = _lib.load()
    scene, sky, params, (w, h) = synthetic.sphere_scene(0, 64, 48)
    k = RendererKernel(scene, sky, params)
    k.update(w, h)
    d_out = torch.full((3,), float("nan"), dtype=torch.float64, device="cuda")
    for _ in range(2):
        k.execute(3)
        expected = k.film_mean()
        film, _ = k.film()
        d_rgb = torch.from_numpy(np.ascontiguousarray(film.reshape(-1))).to("cuda")
        d_out.fill_(float("nan"))
        torch.cuda.synchronize()
        rc = lib.dfpt_film_mean_noalloc(C.c_void_p(d_rgb.data_ptr()), w * h, C.c_void_p(d_out.data_ptr()),
                                        C.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert rc == 0, lib.dfpt_last_error()
        torch.cuda.synchronize()
        np.testing.assert_allclose(d_out.cpu().numpy(), expected, rtol=1e-9, atol=1e-12)
    # Sizes beyond the fixed scratch's limit are rejected before any device work.
    rc = lib.dfpt_film_mean_noalloc(C.c_void_p(d_rgb.data_ptr()), (1 << 28) + 1, C.c_void_p(d_out.data_ptr()), None)
    assert rc == -1 and b"pixel_count" in lib.dfpt_last_error()
    k.dispose()

"""GPU: the L2 read-bandwidth probe bench.py takes its traversal roof from.

A 48 MiB buffer (smaller than L2) streamed through L2 reads faster than the HBM copy rate of the
same GPU and stays within physical limits; a 1 GiB buffer (far larger than L2) reads at most at
DRAM speed.
"""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


def _gbs(lib, buf, repeats, stream):
    g = C.c_double()
    assert lib.dfpt_probe_read_bandwidth(C.c_void_p(buf.data_ptr()), buf.numel() * 4, repeats, C.c_void_p(stream.cuda_stream),
                                         C.byref(g)) == 0
    return g.value


def test_l2_resident_reads_beat_dram_reads(lib):
    import torch

    s = torch.cuda.Stream()
    small = torch.ones(48 * (1 << 20) // 4, device="cuda")
    big = torch.ones((1 << 30) // 4, device="cuda")
    torch.cuda.synchronize()
    l2 = max(_gbs(lib, small, 100, s) for _ in range(3))
    dram = max(_gbs(lib, big, 3, s) for _ in range(2))
    assert 0 < dram < 10000.0, dram  # the HBM3e peak is about 8 TB/s
    assert 1.3 * dram < l2 < 200000.0, (l2, dram)

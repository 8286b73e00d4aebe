"""Host arrays of GpuSim(pinned=True): zeroed, of the requested type and
length, on anonymous memory aligned to the transparent huge page size (the
host link sustains both directions at full rate from huge pages only);
unpinned arrays are plain numpy arrays. No CUDA call is made."""
import numpy as np

from tristan_gb300 import gpu
from tristan_gb300.setups import PARTICLE_DTYPE


def test_pinned_host_arrays_are_zeroed_and_huge_page_aligned():
    huge = gpu._huge_page_bytes()
    assert huge >= 2 << 20 and huge & (huge - 1) == 0
    for n, dt in ((1000, np.float32), (12345, PARTICLE_DTYPE)):
        a = gpu._host_array(n, dt, True)
        assert a.dtype == np.dtype(dt) and a.shape == (n,)
        assert a.ctypes.data % huge == 0
        assert not a.view(np.uint8).any()
        a[-1] = a[0]  # writable to the last element
        assert a.flags.c_contiguous and a.flags.writeable


def test_unpinned_host_arrays_are_plain():
    a = gpu._host_array(10, np.float32, False)
    assert isinstance(a, np.ndarray) and a.shape == (10,) and not a.any()
    assert gpu._host_array(0, np.float32, True).shape == (0,)


def test_huge_page_fraction_reads_the_arrays_mappings():
    a = gpu._host_array(3 * gpu._huge_page_bytes() // 4, np.float32, True)
    a[:] = 1.0  # touch every page
    f = gpu.huge_page_fraction([a])
    assert f is None or 0.0 <= f <= 1.0
    assert gpu.huge_page_fraction([]) is None
    assert gpu.huge_page_fraction([np.zeros(0, np.float32)]) is None

"""gbrkc_advance_noalloc, the advance for callers that must not allocate
device memory while they step (a host whose GPU memory belongs to its own
allocator, or a real-time loop that cannot take the synchronisation of a
cudaMalloc / cudaFree): its launch scratch lives in the library's static
device memory.  It must give exactly what gbrkc_advance gives, call after
call -- the shared scratch keeps the previous call's contents, so two calls
in a row check that what must start at zero is cleared -- and it must leave
the device's free memory unchanged once the first launch has loaded the
kernels.

Collected last on purpose (test_zz_*): a run that stops at its first
failure has run every other test by then.  It passes alone in a fresh
process too (gbrkc_build sets the scratch address up)."""
import ctypes
import ctypes.util
import os

import numpy as np
import pytest

import configs
import gbrkc as G

pytestmark = pytest.mark.gpu


def _cudart():
    """The CUDA runtime shared library, for cudaMemGetInfo (device-wide)."""
    names = [os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64", "libcudart.so"),
             ctypes.util.find_library("cudart") or "libcudart.so"]
    for n in names:
        try:
            rt = ctypes.CDLL(n)
            rt.cudaMemGetInfo.argtypes = [ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]
            return rt
        except OSError:
            continue
    pytest.skip("no CUDA runtime library to read free device memory")


def _free_bytes(rt):
    free, total = ctypes.c_size_t(), ctypes.c_size_t()
    assert rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
    return free.value


@pytest.mark.parametrize("precision", [G.FP64, G.MIXED])
def test_noalloc_advance_matches_advance(precision):
    specs = configs.scaled_mixed_batch(1.0 / 64)
    engines = []
    for _ in range(2):
        eng = G.Engine(precision)
        ids = configs.add_to(eng, specs)
        eng.build()
        engines.append((eng, ids))
    (ref, ids_ref), (new, ids_new) = engines
    persistent, ctas = new.launch_layout()
    assert persistent and sum(ctas) <= 1024, ctas
    t = 0.0
    for call in range(2):
        ref.advance(t, 8, tolerate_retire=True)
        new.advance_noalloc(t, 8, tolerate_stopped=True)
        t += 8 * G.H_MAX
        for k, (a, b) in enumerate(zip(ids_ref, ids_new)):
            # the FP64 path is exact, and scheduling never changes a system's
            # arithmetic in either precision: identical bits
            np.testing.assert_array_equal(new.vnew(b), ref.vnew(a), err_msg=f"call {call} system {k}")
        assert new.compartment_updates(-1) == ref.compartment_updates(-1)
    for eng, _ in engines:
        eng.close()


def test_noalloc_advance_allocates_nothing():
    """Free device memory is the same before and after three more calls --
    one of them right after a slot reset, which makes the call run the init
    launch first -- and the results still equal gbrkc_advance's."""
    rt = _cudart()
    specs = configs.scaled_mixed_batch(1.0 / 64)
    ref, new = G.Engine(G.MIXED), G.Engine(G.MIXED)
    ids_ref, ids_new = configs.add_to(ref, specs), configs.add_to(new, specs)
    ref.build()
    new.build()
    t = 0.0
    # first calls load the kernels (lazy module loading) and size local memory
    ref.advance(t, 4, tolerate_retire=True)
    new.advance_noalloc(t, 4, tolerate_stopped=True)
    t += 4 * G.H_MAX
    free0 = _free_bytes(rt)
    gr = [k for k, s in enumerate(specs) if s.cell_type == G.GR]
    for call in range(3):
        if call == 1:
            # refill the first granule systems with new cells in both engines
            jit = np.linspace(-0.4, 0.4, 4)
            ref.reset_systems(ids_ref[gr[0]], 4, jit)
            new.reset_systems(ids_new[gr[0]], 4, jit)
        ref.advance(t, 4, tolerate_retire=True)
        new.advance_noalloc(t, 4, tolerate_stopped=True)
        t += 4 * G.H_MAX
        assert _free_bytes(rt) == free0, f"call {call}: free device memory changed"
    for a, b in zip(ids_ref, ids_new):
        np.testing.assert_array_equal(new.vnew(b), ref.vnew(a))
    ref.close()
    new.close()

"""gbrkc_advance_noalloc, the advance for callers that must not allocate
device memory while they step (a host whose GPU memory belongs to its own
allocator, or a real-time loop that cannot take the synchronisation of a
cudaMalloc / cudaFree): its launch scratch lives in the library's static
device memory.  It must give exactly what gbrkc_advance gives, call after
call -- the shared scratch keeps the previous call's contents, so two calls
in a row check that what must start at zero is cleared.

Collected last on purpose (test_zz_*): a run that stops at its first
failure has run every other test by then.  It passes alone in a fresh
process too (the first call on the device sets the scratch up)."""
import numpy as np
import pytest

import configs
import gbrkc as G

pytestmark = pytest.mark.gpu


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

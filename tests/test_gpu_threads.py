"""Host-thread concurrency of the C ABI (ctypes releases the GIL during each
call, so the threads really overlap in the library).  Models and batches are
used one per thread (the documented rule) but many at once, each on its own
stream, including the first run of a batch, which captures its CUDA graph
(thread-local capture mode); the server is called from several threads at
once.  Every result must equal the same work done alone, bit for bit."""
import threading

import numpy as np
import pytest

from test_capi_host import earth_model

pytestmark = pytest.mark.gpu

SMALL = (64, 16, 4, 16, 8, 4, 16, 4)
MEDIUM = (128, 32, 8, 32, 16, 8, 32, 8)
HALFISH = (128, 32, 16, 64, 16, 4, 32, 8)
LUTS = ("LUT_TRANSMITTANCE", "LUT_SCATTERING", "LUT_IRRADIANCE")


def run_threads(fn, n, timeout=300.0):
    errors = []

    def wrap(i):
        try:
            fn(i)
        except Exception as e:  # reported after the join
            errors.append((i, e))
    threads = [threading.Thread(target=wrap, args=(i,)) for i in range(n)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout)
    assert not any(t.is_alive() for t in threads), "a thread did not finish"
    assert not errors, errors


def test_models_on_threads_equal_sequential(atmo, torch_cuda):
    torch = torch_cuda
    shapes = [MEDIUM, SMALL, HALFISH, MEDIUM]
    ref = []
    for s in shapes:
        m = earth_model(atmo, shape=s, combined=(s != SMALL))
        m.Init(4)
        ref.append((m.transmittance(), m.scattering(), m.irradiance()))
    models = [earth_model(atmo, shape=s, combined=(s != SMALL)) for s in shapes]
    streams = [torch.cuda.Stream() for _ in shapes]

    def work(i):
        for _ in range(3):
            models[i].Init(4, stream=streams[i])
    run_threads(work, len(shapes))
    for m, (t, s, irr) in zip(models, ref):
        np.testing.assert_array_equal(m.transmittance(), t)
        np.testing.assert_array_equal(m.scattering(), s)
        np.testing.assert_array_equal(m.irradiance(), irr)


def test_batches_capture_and_replay_on_threads(atmo, oracle, torch_cuda):
    torch = torch_cuda
    from test_gpu_parity import random_atmosphere
    rng = np.random.default_rng(5)
    groups = [[random_atmosphere(oracle, rng) for _ in range(3)] for _ in range(4)]
    shapes = [[SMALL, MEDIUM, HALFISH], [MEDIUM] * 3, [HALFISH, SMALL, SMALL], [SMALL] * 3]
    orders = [[2, 4, 3], [3, 3, 5], [4, 2, 2], [6, 3, 4]]
    ref = []
    for g, s, o in zip(groups, shapes, orders):
        b = atmo.Batch(g, s, o)
        b.run()
        atmo.synchronize_stream()
        ref.append([[b.read(i, getattr(atmo, k)) for k in LUTS] for i in range(3)])
    batches = [atmo.Batch(g, s, o) for g, s, o in zip(groups, shapes, orders)]
    streams = [torch.cuda.Stream() for _ in batches]

    def work(i):
        for _ in range(3):      # the first run captures the graph, the others replay it
            batches[i].run(streams[i])
        streams[i].synchronize()
    run_threads(work, len(batches))
    for b, r in zip(batches, ref):
        for i in range(3):
            for k, want in zip(LUTS, r[i]):
                np.testing.assert_array_equal(b.read(i, getattr(atmo, k)), want)


def test_server_called_from_threads(atmo, oracle, torch_cuda):
    atm = oracle.earth_atmosphere()
    alone = atmo.Server()
    t = alone.submit_rebuild(atm, SMALL, 3)
    alone.wait(t)
    want = [alone.lut_set(t).read(getattr(atmo, k)) for k in LUTS]
    alone.close()

    srv = atmo.Server(shade_streams=2)
    got = {}
    lock = threading.Lock()

    def work(i):
        ids = [srv.submit_rebuild(atm, SMALL, 3) for _ in range(4)]
        for t in ids:
            assert srv.wait(t).state == atmo.Server.DONE
            reads = [srv.lut_set(t).read(getattr(atmo, k)) for k in LUTS]
            with lock:
                got[t] = reads
        srv.stats()
    run_threads(work, 4)
    assert len(got) == 16
    for reads in got.values():
        for a, b in zip(reads, want):
            np.testing.assert_array_equal(a, b)
    srv.close()

"""The serving engine (atmo_server_*): rebuilds batched at pass granularity
with uneven LUT shapes and order counts, shading requests beside them, LUT
sets resident under an HBM budget with LRU eviction.  Each result must be the
same alone and in the mix (bit for bit: the kernels assign tiles per
instance), and the same as the standalone batched precomputation."""
import ctypes as C
import time

import numpy as np
import pytest

from test_gpu_parity import random_atmosphere

HALF = (128, 32, 16, 64, 16, 4, 32, 8)
SMALL = (64, 16, 4, 16, 8, 4, 16, 4)
MEDIUM = (128, 32, 8, 32, 16, 8, 32, 8)
LUTS = ("LUT_TRANSMITTANCE", "LUT_SCATTERING", "LUT_IRRADIANCE")


def test_server_needs_a_device(atmo):
    """Without a GPU the server reports the CUDA error instead of running."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(atmo.AtmoError) as e:
        atmo.Server()
    assert e.value.status == atmo.CUDA_ERROR


def test_server_config_limits(atmo):
    """Out-of-range settings are refused before any device work."""
    for kw in ({"max_rebuilds_in_flight": 5000}, {"shade_streams": 65},
               {"admit_window_us": 20000000}):
        with pytest.raises(atmo.AtmoError) as e:
            atmo.Server(**kw)
        assert e.value.status == atmo.INVALID_ARG


def make_view(atmo, seed, width=96, height=54):
    rng = np.random.default_rng(seed)
    cam = rng.normal(size=3)
    cam = cam / np.linalg.norm(cam) * (6360.0 + rng.uniform(0.0, 100.0))
    fwd = rng.normal(size=3)
    fwd /= np.linalg.norm(fwd)
    tmp = rng.normal(size=3)
    right = np.cross(fwd, tmp)
    right /= np.linalg.norm(right)
    up = np.cross(right, fwd)
    sun = rng.normal(size=3)
    sun /= np.linalg.norm(sun)
    v = atmo.PinholeView()
    for name, x in (("camera", cam), ("right", right), ("up", up), ("forward", fwd),
                    ("sun_direction", sun), ("albedo", (0.1, 0.1, 0.1))):
        setattr(v, name, (C.c_float * 3)(*x))
    v.fov_y = np.radians(50.0)
    v.width, v.height = width, height
    depth = rng.uniform(0.1, 100.0, size=width * height).astype(np.float32)
    return v, depth


def shade(torch, server, set_id, view, depth):
    d = torch.from_numpy(depth).cuda()
    sky = torch.empty((view.height, view.width, 4), device="cuda")
    shaded = torch.empty_like(sky)
    t = server.submit_shade(set_id, view, d, sky, shaded)
    return t, (d, sky, shaded)


@pytest.mark.gpu
def test_same_alone_and_in_the_mix(atmo, oracle, torch_cuda):
    torch = torch_cuda
    rng = np.random.default_rng(2024)
    atms = [random_atmosphere(oracle, rng) for _ in range(7)]
    atms.insert(3, oracle.earth_atmosphere())
    shapes = [HALF, SMALL, MEDIUM, atmo.DEFAULT_SHAPE, SMALL, HALF, MEDIUM, SMALL]
    orders = [2, 5, 3, 4, 6, 3, 2, 4]
    key = 3   # the Earth set, compared alone and in the mix
    view, depth = make_view(atmo, 1)

    alone = atmo.Server()
    t = alone.submit_rebuild(atms[key], shapes[key], orders[key])
    alone.wait(t)
    ref = {k: alone.lut_set(t).read(getattr(atmo, k)) for k in LUTS}
    st, bufs = shade(torch, alone, t, view, depth)
    alone.wait(st)
    torch.cuda.synchronize()
    ref_sky, ref_shaded = bufs[1].cpu().numpy(), bufs[2].cpu().numpy()
    alone.close()

    # A batching window long enough that the first five rebuilds, submitted
    # back to back, are admitted together and share their launches; the last
    # three arrive while those run, between shading requests.
    mix = atmo.Server(shade_streams=3, admit_window_us=100000)
    tickets = [mix.submit_rebuild(a, s, o) for a, s, o in zip(atms[:5], shapes[:5], orders[:5])]
    keep = []
    for i, (a, s, o) in enumerate(zip(atms[5:], shapes[5:], orders[5:])):
        # Shading on an earlier set while later rebuilds arrive.
        v2, d2 = make_view(atmo, 100 + i)
        keep.append(shade(torch, mix, tickets[i], v2, d2))
        tickets.append(mix.submit_rebuild(a, s, o))
    key_shade, key_bufs = shade(torch, mix, tickets[key], view, depth)
    for t in tickets:
        mix.wait(t)
    for t, _ in keep:
        assert mix.wait(t).state == atmo.Server.DONE
    mix.wait(key_shade)
    torch.cuda.synchronize()
    for k in LUTS:
        np.testing.assert_array_equal(mix.lut_set(tickets[key]).read(getattr(atmo, k)), ref[k])
    np.testing.assert_array_equal(key_bufs[1].cpu().numpy(), ref_sky)
    np.testing.assert_array_equal(key_bufs[2].cpu().numpy(), ref_shaded)
    stats = mix.stats()
    assert stats.rounds > 0 and stats.kernels >= stats.rounds
    # Some round launched a kernel for more than one instance.
    assert stats.kernels < sum(4 + 3 * (o - 1) for o in orders)

    # The same LUTs as the standalone batched precomputation.
    b = atmo.Batch(atms[:3], shapes[:3], orders[:3])
    b.run()
    atmo.synchronize_stream()
    for i in range(3):
        for k in LUTS:
            np.testing.assert_array_equal(mix.lut_set(tickets[i]).read(getattr(atmo, k)),
                                          b.read(i, getattr(atmo, k)))
    mix.close()


@pytest.mark.gpu
def test_budget_and_lru_eviction(atmo, oracle, torch_cuda):
    torch = torch_cuda
    # SMALL: final LUTs T 64x16 (twice, with the optical depth), I 16x4 and
    # S 4x16x32 texels of 16 B; temporaries: delta irradiance, 3 delta S and
    # the set-up tables (48 B rows, 16 B columns), each rounded up to 256 B.
    final = 64 * 16 * 16 * 2 + 16 * 4 * 16 + 4 * 16 * 32 * 16
    scratch = 16 * 4 * 16 + 3 * 4 * 16 * 32 * 16 + 4 * 16 * 48 + 256 + 4 * 16 * 48 + 256 + 256
    # Room for two ready sets and a third being built (its final LUTs and
    # temporaries), not for three ready sets and a fourth being built.
    budget = int(3.5 * final) + scratch
    srv = atmo.Server(hbm_budget_bytes=budget)
    a = oracle.earth_atmosphere()
    ids = []
    for i in range(3):
        ids.append(srv.submit_rebuild(a, SMALL, 2))
        srv.wait(ids[-1])
    srv.lut_set(ids[0])          # set 0 is now the most recently used
    ids.append(srv.submit_rebuild(a, SMALL, 2))
    srv.wait(ids[-1])
    st = srv.stats()
    assert st.evictions >= 1
    srv.lut_set(ids[0])          # still resident
    with pytest.raises(atmo.AtmoError) as e:
        srv.lut_set(ids[1])      # the least recently used set went first
    assert e.value.status == atmo.NOT_READY
    # A shading request on an evicted set fails with NOT_READY.
    view, depth = make_view(atmo, 3, 16, 8)
    t, bufs = shade(torch, srv, ids[1], view, depth)
    with pytest.raises(atmo.AtmoError) as e:
        srv.wait(t)
    assert e.value.status == atmo.NOT_READY
    # A rebuild larger than the whole budget is refused.
    big = srv.submit_rebuild(a, atmo.DEFAULT_SHAPE, 2)
    with pytest.raises(atmo.AtmoError) as e:
        srv.wait(big)
    assert e.value.status == atmo.BUDGET
    # Explicit eviction frees a ready set.
    srv.evict(ids[0])
    with pytest.raises(atmo.AtmoError):
        srv.lut_set(ids[0])
    srv.close()


@pytest.mark.gpu
def test_destroy_with_work_in_flight(atmo, oracle, torch_cuda):
    """Closing the server while rebuilds and shading requests run returns
    once their GPU work has finished (no hang, no fault)."""
    torch = torch_cuda
    import time
    srv = atmo.Server()
    rng = np.random.default_rng(9)
    ids = [srv.submit_rebuild(random_atmosphere(oracle, rng), MEDIUM, 4) for _ in range(6)]
    keep = []
    view, depth = make_view(atmo, 4)
    for t in ids[:3]:
        keep.append(shade(torch, srv, t, view, depth))
    t0 = time.perf_counter()
    srv.close()
    assert time.perf_counter() - t0 < 60.0
    torch.cuda.synchronize()


@pytest.mark.gpu
def test_pool_that_cannot_serve_an_admitted_rebuild_fails_it_with_oom(atmo, oracle, torch_cuda):
    """The budget admits the rebuild but the private pool, capped below one
    set, cannot serve it: the ticket fails with ATMO_OOM (the allocation
    failure branch of admission), and the server goes on serving requests
    that fit."""
    srv = atmo.Server(pool_max_bytes=32 << 20)
    try:
        t = srv.submit_rebuild(oracle.earth_atmosphere(), atmo.DEFAULT_SHAPE, 4)  # ~65 MB
        with pytest.raises(atmo.AtmoError) as e:
            srv.wait(t, 60000)
        assert e.value.status == atmo.OOM
        info = srv.poll(t)
        assert info.state == atmo.Server.FAILED and info.status == atmo.OOM
        small = srv.submit_rebuild(oracle.earth_atmosphere(), SMALL, 2)            # ~0.3 MB
        assert srv.wait(small, 60000).state == atmo.Server.DONE
        assert srv.stats().used_bytes > 0
    finally:
        srv.close()


@pytest.mark.gpu
def test_wait_times_out_on_a_ticket_held_by_the_batching_window(atmo, oracle, torch_cuda):
    """A lone rebuild waits for company for the batching window (2 s): a wait
    of 50 ms on it returns ATMO_TIMEOUT with the ticket still queued; a
    longer wait then sees it complete."""
    srv = atmo.Server(admit_window_us=2000000)
    try:
        t = srv.submit_rebuild(oracle.earth_atmosphere(), SMALL, 2)
        with pytest.raises(atmo.AtmoError) as e:
            srv.wait(t, 50)
        assert e.value.status == atmo.TIMEOUT
        assert srv.poll(t).state == atmo.Server.QUEUED
        info = srv.wait(t, 60000)
        assert info.state == atmo.Server.DONE
        assert info.queue_ms >= 1900.0            # held by the window
        assert info.rounds == 7 and info.device_ms > 0.0   # 4 + 3 passes, GPU-timed
    finally:
        srv.close()


@pytest.mark.gpu
def test_cancel_a_queued_rebuild_and_its_shading(atmo, oracle, torch_cuda):
    """A rebuild held by the batching window is dropped by cancel; a shading
    request waiting on its set then fails with ATMO_NOT_READY, and a shading
    request still queued can be cancelled itself."""
    torch = torch_cuda
    srv = atmo.Server(admit_window_us=5000000)
    try:
        c = srv.submit_rebuild(oracle.earth_atmosphere(), SMALL, 2)
        view, depth = make_view(atmo, 3)
        s1, keep1 = shade(torch, srv, c, view, depth)
        s2, keep2 = shade(torch, srv, c, view, depth)
        assert srv.poll(c).state == atmo.Server.QUEUED
        srv.cancel(s2)
        srv.cancel(c)
        for t, status in ((c, atmo.CANCELLED), (s2, atmo.CANCELLED), (s1, atmo.NOT_READY)):
            with pytest.raises(atmo.AtmoError) as e:
                srv.wait(t, 10000)
            assert e.value.status == status
        assert srv.stats().used_bytes == 0 and srv.stats().pending == 0
    finally:
        srv.close()


@pytest.mark.gpu
def test_cancel_a_running_rebuild_releases_its_budget(atmo, oracle, torch_cuda):
    """Cancelling a rebuild being built stops it after the passes already
    enqueued and returns its memory to the budget, so a rebuild that did not
    fit beside it is admitted and built; completed tickets cannot be
    cancelled."""
    torch = torch_cuda
    one_set = 70 << 20     # one default-shape set (~65 MB while building) fits, two do not
    srv = atmo.Server(hbm_budget_bytes=one_set)
    try:
        # a: 64 orders (193 passes, tens of ms); b waits for the budget a holds.
        a = srv.submit_rebuild(oracle.earth_atmosphere(), atmo.DEFAULT_SHAPE, 64)
        deadline = time.monotonic() + 10.0
        while srv.poll(a).state == atmo.Server.QUEUED and time.monotonic() < deadline:
            time.sleep(0.0005)
        b = srv.submit_rebuild(oracle.earth_atmosphere(mie_g=0.7), atmo.DEFAULT_SHAPE, 4)
        view, depth = make_view(atmo, 4)
        s_b, keep = shade(torch, srv, b, view, depth)
        assert srv.poll(a).state == atmo.Server.RUNNING
        time.sleep(0.002)
        assert srv.poll(b).state == atmo.Server.QUEUED
        srv.cancel(a)
        with pytest.raises(atmo.AtmoError) as e:
            srv.wait(a, 1000)
        assert e.value.status == atmo.CANCELLED
        # Its budget went back: b is admitted and built, and its shading runs.
        assert srv.wait(b, 60000).state == atmo.Server.DONE
        assert srv.wait(s_b, 60000).state == atmo.Server.DONE
        with pytest.raises(atmo.AtmoError) as e:
            srv.cancel(b)
        assert e.value.status == atmo.INVALID_ARG
        torch.cuda.synchronize()
        st = srv.stats()
        assert st.building == 0 and 0 < st.used_bytes <= one_set
    finally:
        srv.close()


@pytest.mark.gpu
def test_shading_cap_changes_scheduling_not_results(atmo, oracle, torch_cuda):
    """max_shades_in_flight = 1 queues shading on the host: every request
    still completes, with the same pixels as without the cap."""
    torch = torch_cuda
    outs = []
    for cap in (0, 1):
        srv = atmo.Server(max_shades_in_flight=cap)
        try:
            set_id = srv.submit_rebuild(oracle.earth_atmosphere(), SMALL, 3)
            tickets, keep = [], []
            for seed in range(5):
                view, depth = make_view(atmo, 10 + seed)
                t, k = shade(torch, srv, set_id, view, depth)
                tickets.append(t)
                keep.append(k)
            for t in tickets:
                assert srv.wait(t, 60000).state == atmo.Server.DONE
            torch.cuda.synchronize()
            outs.append([torch.cat([k[1].flatten(), k[2].flatten()]) for k in keep])
        finally:
            srv.close()
    for a, b in zip(*outs):
        assert torch.equal(a, b)

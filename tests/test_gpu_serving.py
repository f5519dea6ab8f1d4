"""Serving loop (config 4): continuous batching of per-session frame requests
(GB300 only).

Each result must be the same whether its request ran alone or batched with
other sessions' requests: the batched launch is exact per pixel, so the test
asks for identical bits.
"""
import numpy as np
import pytest

from meteoros_gb300 import abi, scenes
from tests.gpu_util import assert_bits_equal

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SIZES = ((64, 36), (160, 90), (97, 55), (128, 128))


@pytest.fixture(scope="module")
def ctx(lib):
    from meteoros_gb300.renderer import Context

    c = Context(0)
    c.generate_volumes(7)
    c.generate_weather(0, 7)
    yield c
    c.close()


def session_path(i, w, h, frames):
    """Per-frame (camera, time) of session i: yawing 0.5 deg/frame from a seeded start."""
    seq = scenes.config_sequence(100 + i, w, h, frames=frames)
    return [(cam, tm) for cam, _, tm, _ in seq], seq[0][3]


def run_sessions(ctx, n_sessions, frames, mixed, max_batch=64, streams=2, per_request=False, use_graph=False):
    """Renders `frames` requests per session; mixed=False runs one request at a
    time (submit, wait), mixed=True submits every session's next request at
    once, so they batch.  Returns each session's frames as host arrays."""
    from meteoros_gb300.server import Server

    out = {}
    with Server(ctx, max_batch=max_batch, streams=streams, hbm_budget_bytes=1 << 30,
                per_request=per_request, use_graph=use_graph) as srv:
        paths, sids = [], []
        for i in range(n_sessions):
            w, h = SIZES[i % len(SIZES)]
            path, params = session_path(i, w, h, frames)
            sids.append(srv.open_session(w, h, params))
            paths.append(path)
        infos = []
        for f in range(frames):
            if mixed:
                rids = [srv.submit(s, *paths[i][f]) for i, s in enumerate(sids)]
                infos += [srv.wait(r) for r in rids]
            else:
                for i, s in enumerate(sids):
                    infos.append(srv.wait(srv.submit(s, *paths[i][f])))
            for i, s in enumerate(sids):
                out[(i, f)] = srv.read_frame(s)
    return out, infos


def test_result_is_the_same_alone_and_in_the_mix(ctx):
    alone, infos_a = run_sessions(ctx, 6, 3, mixed=False)
    mixed, infos_m = run_sessions(ctx, 6, 3, mixed=True)
    assert max(i.batch_size for i in infos_a) == 1
    assert max(i.batch_size for i in infos_m) > 1
    for key, (rgba, mask) in alone.items():
        assert_bits_equal(mixed[key][0], rgba, f"session {key[0]} frame {key[1]} rgba")
        assert_bits_equal(mixed[key][1], mask, f"session {key[0]} frame {key[1]} mask")
    for i in infos_a + infos_m:
        assert i.status == abi.MT_OK
        assert i.submit_s <= i.start_s <= i.done_s
    # batches captured as CUDA graphs give the same frames
    graphed, infos_g = run_sessions(ctx, 6, 3, mixed=True, use_graph=True)
    for key, (rgba, mask) in alone.items():
        assert_bits_equal(graphed[key][0], rgba, f"session {key[0]} frame {key[1]} rgba (graph)")
        assert_bits_equal(graphed[key][1], mask, f"session {key[0]} frame {key[1]} mask (graph)")
    # the plain per-request launch (mt_render per request) gives the same frames
    plain, infos_p = run_sessions(ctx, 6, 3, mixed=True, streams=1, per_request=True)
    assert max(i.batch_size for i in infos_p) == 1
    for key, (rgba, mask) in alone.items():
        assert_bits_equal(plain[key][0], rgba, f"session {key[0]} frame {key[1]} rgba (per request)")
        assert_bits_equal(plain[key][1], mask, f"session {key[0]} frame {key[1]} mask (per request)")


def test_served_frames_equal_per_view_renders(ctx):
    """A session's frames through the server equal mt_render of the same
    uniforms: frame 0 full, later frames checkerboard over the previous one."""
    from meteoros_gb300.server import Server

    w, h = 97, 55
    path, params = session_path(3, w, h, 3)
    with Server(ctx, hbm_budget_bytes=1 << 30) as srv:
        sid = srv.open_session(w, h, params)
        prev = None
        old = path[0][0]
        for f, (cam, tm) in enumerate(path):
            srv.wait(srv.submit(sid, cam, tm))
            got, gmask = srv.read_frame(sid)
            cur = torch.full((h, w, 4), float("nan"), dtype=torch.float32, device="cuda")
            mask = torch.full((h, w), float("nan"), dtype=torch.float32, device="cuda")
            flags = abi.MT_RENDER_FULL if f == 0 else abi.MT_RENDER_CHECKERBOARD
            if f == 0:
                mask.zero_()
            else:
                mask.copy_(torch.from_numpy(prev_mask))
            ctx.render(cam, old, tm, params, prev, cur, mask, flags)
            torch.cuda.synchronize()
            assert_bits_equal(got, cur.cpu().numpy(), f"frame {f} rgba")
            if f > 0:
                assert_bits_equal(gmask, mask.cpu().numpy(), f"frame {f} mask")
            prev, old, prev_mask = cur, cam, gmask


def test_admission_by_hbm_budget(ctx):
    from meteoros_gb300.server import Server

    _, _, params, _ = scenes.config_view(1, 640, 360)
    per_session = 640 * 360 * (2 * 16 + 4)
    with Server(ctx, hbm_budget_bytes=3 * per_session + 100) as srv:
        sids = [srv.open_session(640, 360, params) for _ in range(3)]
        with pytest.raises(abi.MeteorosError) as e:
            srv.open_session(640, 360, params)
        assert e.value.status == abi.MT_ERR_BUDGET
        assert srv.memory() == (3 * per_session, 3 * per_session + 100)
        srv.close_session(sids[0])
        sids[0] = srv.open_session(640, 360, params)  # room again
        with pytest.raises(abi.MeteorosError):
            srv.submit(12345, *session_path(0, 640, 360, 1)[0][0])


def test_continuous_batching_overlaps_batches(ctx):
    """Requests that arrive while a batch runs join the next one; with two
    streams, a batch starts before the previous one is done."""
    from meteoros_gb300.server import Server

    n = 48
    with Server(ctx, max_batch=8, streams=2, hbm_budget_bytes=1 << 30) as srv:
        sids, paths = [], []
        for i in range(n):
            path, params = session_path(i, 320, 180, 2)
            sids.append(srv.open_session(320, 180, params))
            paths.append(path)
        for f in range(2):
            rids = [srv.submit(s, *paths[i][f]) for i, s in enumerate(sids)]
            infos = [srv.wait(r) for r in rids]
        assert max(i.batch_size for i in infos) <= 8
        batches = sorted({(i.start_s, i.done_s) for i in infos})
        assert len(batches) >= n // 8
        overlapped = any(b[0] < a[1] for a, b in zip(batches, batches[1:]))
        assert overlapped, "no batch started while the previous one ran"


def test_admission_waits_for_budget_to_free(ctx):
    """With admission_wait_ms, a session that does not fit is admitted once a
    closing session frees the budget; without a close it fails after the wait."""
    import threading
    import time

    from meteoros_gb300.server import Server

    _, _, params, _ = scenes.config_view(2, 320, 180)
    per_session = 320 * 180 * (2 * 16 + 4)
    with Server(ctx, hbm_budget_bytes=2 * per_session, admission_wait_ms=3000) as srv:
        a = srv.open_session(320, 180, params)
        srv.open_session(320, 180, params)
        closer = threading.Timer(0.2, lambda: srv.close_session(a))
        t0 = time.perf_counter()
        closer.start()
        srv.open_session(320, 180, params)  # waits for the close
        waited = time.perf_counter() - t0
        closer.join()
        assert 0.1 < waited < 3.0
    with Server(ctx, hbm_budget_bytes=per_session, admission_wait_ms=100) as srv:
        srv.open_session(320, 180, params)
        with pytest.raises(abi.MeteorosError) as e:
            srv.open_session(320, 180, params)
        assert e.value.status == abi.MT_ERR_BUDGET


def test_concurrent_close_read_and_wait(ctx):
    """Several host threads close, read and wait on the same sessions and
    requests at once while others open sessions (inserts that rehash the
    server's maps): every call returns a defined status -- one close of a
    session succeeds, the others report an unknown or meanwhile-closed
    session; one wait on a request takes it, the other reports it unknown."""
    import ctypes as C
    import threading

    from meteoros_gb300.server import Server

    lib = ctx.lib
    _, _, params, _ = scenes.config_view(5, 160, 90)
    for rnd in range(4):
        with Server(ctx, max_batch=8, streams=2, hbm_budget_bytes=1 << 30) as srv:
            h = srv.handle
            sids = [srv.open_session(160, 90, params) for _ in range(12)]
            path = session_path(rnd, 160, 90, 1)[0]
            rids = [srv.submit(s, *path[0]) for s in sids]
            results = {"close": [], "read": [], "wait": [], "open": []}
            lock = threading.Lock()
            rgba = np.empty((90, 160, 4), np.float32)

            def close(s):
                st = lib.mt_server_close_session(h, C.c_int64(s))
                with lock:
                    results["close"].append((s, st))

            def read(s):
                buf = np.empty_like(rgba)
                st = lib.mt_server_read_frame(h, C.c_int64(s), buf.ctypes.data_as(C.c_void_p), None)
                with lock:
                    results["read"].append((s, st))

            def wait(r):
                info = abi.RequestInfo()
                st = lib.mt_server_wait(h, C.c_uint64(r), 30000, C.byref(info))
                with lock:
                    results["wait"].append((r, st))

            def opener():
                for _ in range(64):  # grows the session map past several rehashes
                    sid = C.c_int64()
                    st = lib.mt_server_open_session(h, 16, 16, C.byref(params), C.byref(sid))
                    with lock:
                        results["open"].append(st)

            threads = [threading.Thread(target=opener)]
            for s, r in zip(sids, rids):
                threads += [threading.Thread(target=wait, args=(r,)), threading.Thread(target=wait, args=(r,)),
                            threading.Thread(target=read, args=(s,)), threading.Thread(target=close, args=(s,)),
                            threading.Thread(target=close, args=(s,))]
            for t in threads:
                t.start()
            for t in threads:
                t.join(60)
            assert not any(t.is_alive() for t in threads)
            assert all(st == abi.MT_OK for st in results["open"])
            for s in sids:
                sts = sorted(st for x, st in results["close"] if x == s)
                assert sts == [abi.MT_OK, abi.MT_ERR_INVALID_ARG], (s, sts)
            for s, st in results["read"]:
                assert st in (abi.MT_OK, abi.MT_ERR_INVALID_ARG, abi.MT_ERR_NO_VOLUMES), (s, st)
            for r in rids:
                sts = sorted(st for x, st in results["wait"] if x == r)
                # the request may be failed (INVALID_ARG) when its session closed before it ran
                assert sts.count(abi.MT_ERR_INVALID_ARG) >= 1 and len(sts) == 2, (r, sts)
                assert all(st in (abi.MT_OK, abi.MT_ERR_INVALID_ARG) for st in sts), (r, sts)

"""Serving (rgdn_server_*): continuous batching of frame requests from many camera streams.

A frame's results are the same whether its stream is served alone or in a mix of streams of
other sizes whose frames arrive concurrently from other threads (bit for bit: every batched
step computes each frame exactly as the single-stream path does). Admission under the
context's memory budget and the drop policy for stale frames are checked deterministically.
"""
import threading
import time

import numpy as np
import pytest

from raytracedgl1_gb300 import _native as N
from raytracedgl1_gb300.denoiser import Context, Server, required_bytes
from raytracedgl1_gb300.scene import Scene

pytestmark = pytest.mark.gpu


def host_request(sid, bufs, p, out=None):
    keep = {n: np.ascontiguousarray(a) for n, a in bufs.items()}
    req = Server.request(sid, p, {n: a.ctypes.data for n, a in keep.items()}, N.REQUEST_COPY,
                         out.ctypes.data if out is not None else None)
    return req, keep


def pre_final_bytes(W, H, storage):
    return W * H * {N.STORAGE_REF: 4, N.STORAGE_FP32: 16, N.STORAGE_FP16: 8, N.STORAGE_BF16: 8}[storage]


@pytest.mark.parametrize("storage", [N.STORAGE_FP16, N.STORAGE_REF])
def test_frame_same_alone_and_in_mix(storage):
    ctx = Context(0)
    W, H = 64, 36
    frames = [Scene(W, H, seed=90).generate(f) for f in range(8)]

    def run_main(server, sid, background=None):
        outs = []
        for f, (bufs, p) in enumerate(frames):
            out = np.zeros(pre_final_bytes(W, H, storage), dtype=np.uint8)
            req, keep = host_request(sid, bufs, p, out)
            t = server.submit(req)
            r = server.wait(t)
            assert r.state == N.FRAME_DONE and r.frameIndex == f % 2
            hist, avg, _ = server.stream(sid).tonemapping()
            outs.append((out, hist, avg))
            del keep
        return outs

    with Server(ctx, storage) as alone:
        ref = run_main(alone, alone.open_stream(W, H))

    with Server(ctx, storage, max_frames_per_step=4, steps_in_flight=3) as mix:
        sid = mix.open_stream(W, H)
        others = [(mix.open_stream(w, h), Scene(w, h, seed=91 + i))
                  for i, (w, h) in enumerate([(48, 30), (96, 54), (34, 17), (130, 9), (64, 36)])]
        stop = threading.Event()
        errors = []

        def feeder(k):
            try:
                f = 0
                while not stop.is_set():
                    for j, (osid, sc) in enumerate(others):
                        if j % 2 != k:
                            continue
                        bufs, p = sc.generate(f)
                        p.atrousIterations = 3 + (j + f) % 3
                        if j == 3:
                            p.flags |= N.FLAG_SKIP_GRADIENTS
                        req, keep = host_request(osid, bufs, p)
                        t = mix.submit(req)
                        mix.wait(t)
                        del keep
                    f += 1
            except Exception as e:   # surfaced by the main thread
                errors.append(e)

        threads = [threading.Thread(target=feeder, args=(k,)) for k in range(2)]
        for th in threads:
            th.start()
        time.sleep(0.05)
        got = run_main(mix, sid)
        stop.set()
        for th in threads:
            th.join()
        assert not errors, errors
        st = mix.stats()
        assert st["framesDone"] >= len(frames) + 5 and st["framesDropped"] == 0
    for f, ((oa, ha, aa), (ob, hb, ab)) in enumerate(zip(ref, got)):
        assert np.array_equal(oa, ob), f"frame {f}: PRE_FINAL differs between alone and in the mix"
        assert np.array_equal(ha, hb) and aa == ab, f"frame {f}: tonemapping differs"
    ctx.close()


def test_admission_waits_for_memory():
    W, H = 64, 36
    per = required_bytes(W, H, N.STORAGE_FP16)
    ctx = Context(0, memory_budget_bytes=2 * per + per // 2)   # room for two streams
    sc = Scene(W, H, seed=95)
    bufs, p = sc.generate(0)
    with Server(ctx, N.STORAGE_FP16) as sv:
        ids = [sv.open_stream(W, H) for _ in range(3)]
        keeps, tickets = [], []
        for sid in ids:
            req, keep = host_request(sid, bufs, p)
            keeps.append(keep)
            tickets.append(sv.submit(req))
        for t in tickets[:2]:
            assert sv.wait(t).state == N.FRAME_DONE
        # the third stream does not fit: its frame waits
        with pytest.raises(N.RgdnError) as e:
            sv.drain()
        assert e.value.status == N.OUT_OF_BUDGET
        with pytest.raises(N.RgdnError) as e:
            sv.wait(tickets[2], timeout_ms=50)
        assert e.value.status == N.TIMEOUT
        assert sv.stats()["residentStreams"] == 2
        sv.close_stream(ids[0])                   # frees memory: the third is admitted
        assert sv.wait(tickets[2]).state == N.FRAME_DONE
        sv.drain()
    ctx.close()


def test_stale_frames_are_dropped():
    W, H = 48, 30
    per = required_bytes(W, H, N.STORAGE_FP16)
    ctx = Context(0, memory_budget_bytes=per + per // 2)       # room for one stream
    sc = Scene(W, H, seed=96)
    frames = [sc.generate(f) for f in range(4)]
    with Server(ctx, N.STORAGE_FP16, max_queued_per_stream=1) as sv:
        a, b = sv.open_stream(W, H), sv.open_stream(W, H)
        req, keep_a = host_request(a, *frames[0])
        assert sv.wait(sv.submit(req)).state == N.FRAME_DONE
        # b cannot be admitted while a holds the memory: its frames queue, newer ones win
        keeps, tickets = [], []
        for f in range(1, 4):
            req, keep = host_request(b, *frames[f])
            keeps.append(keep)
            tickets.append(sv.submit(req))
        assert [sv.wait(t).state for t in tickets[:2]] == [N.FRAME_DROPPED, N.FRAME_DROPPED]
        sv.close_stream(a)
        r = sv.wait(tickets[2])
        assert r.state == N.FRAME_DONE and r.frameIndex == 0
        assert sv.stats()["framesDropped"] == 2
    ctx.close()


def test_sm_host_copy_equals_copy_engine():
    """RGDN_HOST_COPY_SM: the planes of requests in pinned host memory are loaded by one kernel
    per frame instead of the copy engines. The results are the same bit for bit, and the kernel
    runs (one launch more per frame). The 130x36 frame's 1-byte IS_SKY plane (4680 bytes, not a
    multiple of 16) still goes through cudaMemcpyAsync."""
    torch = pytest.importorskip("torch")
    ctx = Context(0)
    W, H = 130, 36
    frames = [Scene(W, H, seed=95).generate(f) for f in range(6)]
    pinned = [({n: torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1)).pin_memory() for n, a in b.items()}, p)
              for b, p in frames]
    results, launches = {}, {}
    for mode in (N.HOST_COPY_ENGINE, N.HOST_COPY_SM):
        outs = []
        before = ctx.launch_count()
        with Server(ctx, N.STORAGE_FP16, host_copy=mode) as sv:
            sid = sv.open_stream(W, H)
            for b, p in pinned:
                out = torch.zeros(pre_final_bytes(W, H, N.STORAGE_FP16), dtype=torch.uint8).pin_memory()
                req = Server.request(sid, p, {n: t.data_ptr() for n, t in b.items()}, N.REQUEST_COPY, out.data_ptr())
                r = sv.wait(sv.submit(req))
                assert r.state == N.FRAME_DONE
                hist, avg, _ = sv.stream(sid).tonemapping()
                outs.append((out.numpy().copy(), hist.copy(), avg))
        launches[mode] = ctx.launch_count() - before
        results[mode] = outs
    for f, ((oa, ha, aa), (ob, hb, ab)) in enumerate(zip(results[N.HOST_COPY_ENGINE], results[N.HOST_COPY_SM])):
        assert np.array_equal(oa, ob), f"frame {f}: PRE_FINAL differs"
        assert np.array_equal(ha, hb) and aa == ab, f"frame {f}: tonemapping differs"
    assert launches[N.HOST_COPY_SM] - launches[N.HOST_COPY_ENGINE] == len(frames)
    ctx.close()


@pytest.mark.parametrize("host_copy", [N.HOST_COPY_SM, N.HOST_COPY_ENGINE])
def test_copy_host_planes(host_copy):
    """rgdn_copy_host_planes: pinned (device-mapped) ranges, one of a size that is not a multiple
    of 16 and one in pageable memory (both of which take cudaMemcpyAsync), all land byte for byte;
    bad arguments are refused before any copy."""
    torch = pytest.importorskip("torch")
    from raytracedgl1_gb300.denoiser import copy_host_planes
    rng = np.random.default_rng(3 + host_copy)
    sizes = [1 << 20, (3 << 20) + 16, 4096 + 8, 777 * 16]
    srcs = [torch.from_numpy(rng.integers(0, 256, n, dtype=np.uint8)).pin_memory() for n in sizes[:3]]
    pageable = rng.integers(0, 256, sizes[3], dtype=np.uint8)
    dsts = [torch.zeros(n, dtype=torch.uint8, device="cuda:0") for n in sizes]
    s = torch.cuda.Stream()
    copies = [(d.data_ptr(), h.data_ptr(), n) for d, h, n in zip(dsts[:3], srcs, sizes[:3])]
    copies.append((dsts[3].data_ptr(), pageable.ctypes.data, sizes[3]))
    copy_host_planes(copies, host_copy, s)
    s.synchronize()
    for d, h in zip(dsts[:3], srcs):
        assert torch.equal(d.cpu(), h)
    assert np.array_equal(dsts[3].cpu().numpy(), pageable)
    with pytest.raises(N.RgdnError):
        copy_host_planes([(0, srcs[0].data_ptr(), 16)], host_copy, s)
    with pytest.raises(N.RgdnError):
        copy_host_planes([(dsts[0].data_ptr(), srcs[0].data_ptr(), 16)], 7, s)

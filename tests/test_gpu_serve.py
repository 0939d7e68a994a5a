"""Asynchronous submission, the multi-stream server and its trackers.

The server's contract: frames admitted into slots as they arrive overlap on
the GPU, and each frame's result is the same in the mix as alone (the
kernels are deterministic, so bit for bit).  The tracker is checked against
its CPU restatement (oracle/tracker.py) on the frames where it is a smooth
function of its inputs (start and first update; later frames resample).
"""
import numpy as np
import pytest

from oracle import tracker as TR

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup(tmp_path_factory):
    import geye_gb300 as g
    from geye_gb300 import synth
    d = str(tmp_path_factory.mktemp("models"))
    ctx = g.Context(0, conv=g.CONV_BF16)
    models = [g.Model(ctx, *synth.write_model_csv(s, d)) for s in (synth.CAR_SPEC, synth.PERSON_SPEC)]
    yield g, synth, ctx, models
    for m in models:
        m.close()
    ctx.close()


def same(a, b):
    return all(x["num"] == y["num"] and all(np.array_equal(x[k], y[k]) for k in ("point", "or_point", "type", "scale", "score"))
               for x, y in zip(a, b))


def test_submit_collect_matches_detect_multi(setup):
    g, synth, ctx, models = setup
    frame = synth.make_frame(640, 480, seed=4)
    ref = ctx.detect_multi(frame, models, -0.5, 0.5, None)
    ctx.detect_submit(frame, models, -0.5, 0.5)
    while not ctx.detect_done():
        pass
    assert same(ctx.detect_collect(), ref)


def test_server_results_same_in_the_mix_as_alone(setup):
    g, synth, ctx, models = setup
    sizes = [(320, 240), (640, 480), (320, 240), (640, 480), (640, 480), (320, 240)]
    frames = {(s, k): synth.make_frame(*sizes[s], seed=10 * s + k) for s in range(len(sizes)) for k in range(2)}
    alone = {key: ctx.detect_multi(f, models, -0.5, 0.5, None) for key, f in frames.items()}
    with g.Server(models, conv=g.CONV_BF16, max_slots=4) as srv:
        tickets = {}
        for k in range(2):
            for s in range(len(sizes)):
                tickets[srv.submit(s, frames[(s, k)])] = (s, k)
        srv.drain()
        done = srv.poll(64)
        assert len(done) == len(frames)
        for d in done:
            assert same(d["results"], alone[tickets[d["ticket"]]])
            assert d["latency_ns"] >= d["queued_ns"] >= 0
        st = srv.stats()
        assert 1 <= st["slots"] <= 4 and st["completed"] == len(frames) and st["queued"] == 0


def test_server_admission_respects_the_memory_budget(setup):
    g, synth, ctx, models = setup
    with g.Server(models, conv=g.CONV_BF16, hbm_budget=1, max_slots=8) as srv:
        for k in range(5):
            srv.submit(k, synth.make_frame(320, 240, seed=k))
        srv.drain()
        assert len(srv.poll(16)) == 5
        assert srv.stats()["slots"] == 1   # the first slot's plan already exceeds the budget


def _dets(results):
    return np.concatenate([r["point"].astype(np.float64).reshape(-1, 4) for r in results])


def test_tracker_matches_its_restatement_and_isolates_streams(setup):
    g, synth, ctx, models = setup
    seq0 = [synth.make_frame(320, 240, seed=100 + k) for k in range(3)]
    seq1 = [synth.make_frame(320, 240, seed=200 + k) for k in range(2)]
    with g.Server(models, conv=g.CONV_BF16, max_slots=3, track=True) as mix:
        order = [(0, seq0[0]), (1, seq1[0]), (0, seq0[1]), (1, seq1[1]), (0, seq0[2])]
        tk = {mix.submit(s, f): s for s, f in order}
        mix.drain()
        done = sorted(mix.poll(16), key=lambda d: d["ticket"])
        tracks_mix = mix.tracks(0)
    with g.Server(models, conv=g.CONV_BF16, max_slots=1, track=True) as solo:
        ref = TR.StreamTracker(0)
        for k, f in enumerate(seq0):
            solo.submit(0, f)
            solo.drain()
            d = solo.poll(4)[0]
            # the frame's A_SCORE maps (same conv mode, fresh -100 start, as the server's)
            asc = [np.full((320, 240), -100, np.float32) for _ in models]
            ctx.detect_multi(f, models, -0.5, 0.5, asc)
            ref.step(_dets(d["results"])[:TR.MAX_DET], np.stack(asc))
            got = solo.tracks(0)
            assert d["n_tracks"] == len(got) == len(ref.boxes())
            if k < 2:   # start and first update: no resampling has happened yet
                assert np.allclose(got, ref.boxes(), rtol=0, atol=0.05), np.abs(got - ref.boxes()).max()
        tracks_solo = solo.tracks(0)
    assert [tk[d["ticket"]] for d in done] == [0, 1, 0, 1, 0]
    assert np.array_equal(tracks_mix, tracks_solo)   # stream 1 did not disturb stream 0


@pytest.mark.parametrize("conv", ["fp32", "bf16"])
def test_batch_graph_matches_single_frames(tmp_path, conv):
    """A batch of mixed sizes as one CUDA graph gives each frame's single-frame result."""
    import geye_gb300 as g
    from geye_gb300 import synth
    mode = {"fp32": g.CONV_FP32, "bf16": g.CONV_BF16}[conv]
    sizes = [(320, 240), (640, 480), (320, 240), (400, 300), (640, 480)]
    frames = [synth.make_frame(w, h, seed=50 + i) for i, (w, h) in enumerate(sizes)]
    with g.Context(0, conv=mode) as c:
        ms = [g.Model(c, *synth.write_model_csv(s, str(tmp_path))) for s in (synth.CAR_SPEC, synth.PERSON_SPEC)]
        alone = [c.detect_multi(f, ms, -0.5, 0.5, None) for f in frames]
        with g.Batch(ms, conv=mode, max_frames=8) as b:
            for rep in range(2):   # the second run replays the same graph
                got = b.run(frames)
                for ra, rb in zip(alone, got):
                    for x, y in zip(ra, rb):
                        assert x["num"] == y["num"]
                        for k in ("point", "or_point", "type", "scale", "score"):
                            assert np.array_equal(x[k], y[k]), k
            st = b.stats()
            assert st["lanes"] == len(frames) and st["graphs"] == 1 and st["kernels"] > 0 and st["last_ms"] > 0
        for m in ms:
            m.close()


def test_server_per_stream_queue_cap_drops_stale_frames(tmp_path):
    """One slot, FP32 1080p frames (several ms each): frames of one stream
    submitted while the slot is busy replace each other in the queue; the first
    and the newest are served, the ones in between come back dropped."""
    import geye_gb300 as g
    from geye_gb300 import synth
    with g.Context(0) as c:
        ms = [g.Model(c, *synth.write_model_csv(synth.CAR_SPEC, str(tmp_path)))]
        frames = [synth.make_frame(1920, 1080, seed=70 + k) for k in range(5)]
        with g.Server(ms, conv=g.CONV_FP32, max_slots=1) as srv:
            srv.set_admission(max_queued_per_stream=1)
            tickets = [srv.submit(0, f) for f in frames]
            srv.drain()
            done = {d["ticket"]: d for d in srv.poll(16)}
            assert sorted(done) == tickets
            assert not done[tickets[0]]["dropped"] and not done[tickets[-1]]["dropped"]
            dropped = [t for t in tickets if done[t]["dropped"]]
            assert 1 <= len(dropped) <= 3 and srv.stats()["dropped"] == len(dropped)
            for t in dropped:
                assert all(r["num"] == 0 for r in done[t]["results"])
            alone = c.detect_multi(frames[-1], ms, -0.5, 0.5, None)
            assert same(done[tickets[-1]]["results"], alone)
        for m in ms:
            m.close()


def test_server_refuses_queued_frames_once_a_models_context_is_gone(tmp_path):
    """Destroying the context that loaded a model frees its filters: queued frames
    are dropped and the call reports GEYE_ERR_ARG before anything is launched;
    the frame already on the GPU finishes first (the destroy waits for it)."""
    import geye_gb300 as g
    from geye_gb300 import synth
    load = g.Context(0)
    ms = [g.Model(load, *synth.write_model_csv(synth.CAR_SPEC, str(tmp_path)))]
    frames = [synth.make_frame(1920, 1080, seed=80 + k) for k in range(4)]
    with g.Server(ms, conv=g.CONV_FP32, max_slots=1) as srv:
        tickets = [srv.submit(0, f) for f in frames]
        queued = srv.stats()["queued"]
        load.close()
        if queued:
            with pytest.raises(g.GeyeError):
                srv.poll(16)
        done = {d["ticket"]: d for d in srv.poll(16)}
        srv.drain()
        done.update({d["ticket"]: d for d in srv.poll(16)})
        assert sorted(done) == tickets
        assert sum(d["dropped"] for d in done.values()) == queued >= 1
        with pytest.raises(g.GeyeError):
            srv.submit(0, frames[0])

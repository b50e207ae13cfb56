"""Served preview loop: the scheduling and admission policy on the dry server
(host only), and the GPU server against the stand-alone render entry point.

The policy follows crates/engine/src/coordinator/scheduler.rs: a pending
request is replaced by a later revision (or the same revision submitted later)
and an older one is dropped; the reference's reservations
(crates/gpu/src/memory.rs:44-60) become the admission budget.
"""

import time

import numpy as np
import pytest

from rohditor_gb300 import CaptureContract, ColorContract, OpticsExecution, SensorDescription, clip_levels
from rohditor_gb300 import OutputSpec
from rohditor_gb300.served import DEVELOP, EDIT, EXPORT, PreviewServer

RD_OK, RD_CANCELLED, RD_OVER_BUDGET = 0, 1, 3
MB = 1 << 20


def _image(w=1024, h=1024, seed=0):
    rng = np.random.default_rng(seed)
    raw = rng.integers(300, 4000, size=(h, w), dtype=np.uint16)
    wb = (2.0, 1.0, 1.6)
    desc = SensorDescription(w, h, cfa="RGGB", black=(256.0,), white=(4095.0,), highlight="clip",
                             clip_levels=clip_levels(1.0, wb), demosaic="amaze", demosaic_balance=wb)
    cap = CaptureContract(amount=0.5, radius=0.7, noise_protection=0.5, ceilings=clip_levels(1.0, wb), iterations=8)
    optics = OpticsExecution(w, h)
    return raw, desc, cap, optics, wb


def _footprint(w, h, tw, th):
    """Resident bytes of one image and the develop's transient, as the server charges them."""
    layers = 2 * w * h + 12 * w * h + 12 * tw * th + (3 * tw * th + 8192)
    develop = 32 * w * h + 64 * MB
    return layers, develop


CAM = (1, 0, 0, 0, 1, 0, 0, 0, 1)


def _open(server, image_id, target=(512, 512), seed=0):
    raw, desc, cap, optics, wb = _image(seed=seed)
    return server.open(image_id, raw, desc, cap, optics, target, wb, CAM)


def _edit(ev):
    return ColorContract(wb_gains=(1.0, 1.0, 1.0), camera_to_rec2020=CAM, exposure_ev=ev)


def _results(server, wait_ms=2000):
    server.drain(wait_ms)
    return server.poll(1024)


def test_dry_open_develops_then_edits_render():
    s = PreviewServer.dry(develop_us=1000, render_us=100)
    for i in range(3):
        _open(s, i, seed=i)
    res = _results(s)
    assert sorted(r["image_id"] for r in res if r["kind"] == DEVELOP) == [0, 1, 2]
    assert all(r["status"] == RD_OK for r in res)
    for i in range(3):
        s.submit_edit(i, 1, _edit(0.1 * (i + 1)))
    res = _results(s)
    edits = [r for r in res if r["kind"] == EDIT]
    assert len(edits) == 3 and all(r["status"] == RD_OK for r in edits)
    assert all(r["latency_ms"] >= r["service_ms"] >= 0.0 for r in edits)
    for i in range(3):
        out, hist, rev = s.read_output(i)
        assert rev == 1 and out[0, 0] == int(np.float32(0.1 * (i + 1)) * np.float32(10.0))
        assert hist.sum() == 512 * 512
    st = s.stats()
    assert st["completed"] == 6 and st["failed"] == 0
    s.close()


def test_dry_newest_wins_per_image():
    # While the first develop runs, five edits of one image arrive: only the newest renders.
    s = PreviewServer.dry(develop_us=200_000, render_us=100)
    _open(s, 7)
    ids = [s.submit_edit(7, rev, _edit(0.1 * rev)) for rev in range(1, 6)]
    res = _results(s, 5000)
    by_id = {r["request_id"]: r for r in res}
    assert [by_id[i]["status"] for i in ids[:-1]] == [RD_CANCELLED] * 4
    assert by_id[ids[-1]]["status"] == RD_OK
    assert s.read_output(7)[2] == 5
    assert s.stats()["coalesced"] == 4
    s.close()


def test_dry_older_revision_is_dropped():
    s = PreviewServer.dry(develop_us=200_000, render_us=100)
    _open(s, 1)
    newer = s.submit_edit(1, 9, _edit(0.9))
    older = s.submit_edit(1, 3, _edit(0.3))  # arrives later, but an older revision
    res = {r["request_id"]: r for r in _results(s, 5000)}
    assert res[older]["status"] == RD_CANCELLED and res[newer]["status"] == RD_OK
    assert s.read_output(1)[2] == 9
    s.close()


def test_dry_edits_of_many_images_render_in_one_batch():
    s = PreviewServer.dry(develop_us=1000, render_us=100)
    for i in range(8):
        _open(s, i, seed=i)
    _results(s)
    # While one edit renders (slowly), edits of seven other images arrive: the
    # render lane takes them together as soon as it is free.
    s.lib.rd_server_set_dry_timing(s.handle, 1000, 100_000)
    s.submit_edit(0, 1, _edit(0.2))
    time.sleep(0.03)
    for i in range(1, 8):
        s.submit_edit(i, 1, _edit(0.2))
    res = _results(s, 5000)
    edits = [r for r in res if r["kind"] == EDIT and r["status"] == RD_OK]
    assert len(edits) == 8
    assert sorted(r["batch_size"] for r in edits) == [1] + [7] * 7
    assert s.stats()["batches"] == 2
    s.close()


def test_dry_edit_is_not_held_behind_a_develop():
    s = PreviewServer.dry(develop_us=1000, render_us=100)
    _open(s, 0)
    _open(s, 1, seed=1)
    _results(s)
    s.lib.rd_server_set_dry_timing(s.handle, 300_000, 100)
    raw, desc, cap, optics, wb = _image()
    s.submit_develop(0, 1, cap, optics)
    time.sleep(0.02)
    edit = s.submit_edit(1, 1, _edit(0.3))
    res = {r["request_id"]: r for r in s.poll(16, wait_ms=200)}
    assert edit in res and res[edit]["status"] == RD_OK and res[edit]["latency_ms"] < 100.0
    s.drain(5000)
    s.close()


def test_dry_admission_evicts_least_recently_used():
    layers, develop = _footprint(1024, 1024, 512, 512)
    budget = develop + 2 * layers + MB  # two resident images plus one develop in flight
    s = PreviewServer.dry(budget_bytes=budget, develop_us=1000, render_us=100)
    for i in range(3):
        _open(s, i, seed=i)
        _results(s)
    st = s.stats()
    assert st["evictions"] >= 1 and st["peak_resident_bytes"] <= budget
    # Editing every image re-develops the evicted ones; everything still completes.
    for i in range(3):
        s.submit_edit(i, 1, _edit(0.5))
        res = _results(s)
        assert [r["status"] for r in res if r["kind"] == EDIT] == [RD_OK]
    st = s.stats()
    assert st["redeveloped"] >= 1 and st["failed"] == 0 and st["peak_resident_bytes"] <= budget
    s.close()


def test_dry_request_that_cannot_fit_fails_over_budget():
    layers, develop = _footprint(1024, 1024, 512, 512)
    s = PreviewServer.dry(budget_bytes=develop // 2, develop_us=1000, render_us=100)
    rid = _open(s, 0)
    res = {r["request_id"]: r for r in _results(s)}
    assert res[rid]["status"] == RD_OVER_BUDGET
    s.close()


def test_dry_close_cancels_pending_requests():
    s = PreviewServer.dry(develop_us=200_000, render_us=100)
    _open(s, 0)
    _open(s, 1)
    edit = s.submit_edit(1, 1, _edit(0.1))
    s.close_image(1)
    res = {r["request_id"]: r for r in _results(s, 5000)}
    assert res[edit]["status"] == RD_CANCELLED
    assert s.stats()["resident_bytes"] > 0  # image 0 stays
    s.close()


EXPORTS = [OutputSpec(format="srgb8"), OutputSpec(format="extended_f16", primaries="display_p3",
                                                  policy="chroma_compress", headroom=4.0)]


def test_dry_export_fills_the_client_buffers():
    s = PreviewServer.dry(develop_us=1000, render_us=100)
    _open(s, 3)
    _results(s)
    rid, outs = s.submit_export(3, 1, _edit(0.7), EXPORTS)
    res = {r["request_id"]: r for r in _results(s)}
    assert res[rid]["kind"] == EXPORT and res[rid]["status"] == RD_OK
    assert outs[0].shape == (1024, 3 * 1024) and outs[1].dtype == np.float16
    assert np.all(outs[0] == 7)
    assert s.stats()["exports"] == 1
    s.close()


def test_dry_newer_export_replaces_a_pending_one():
    s = PreviewServer.dry(develop_us=200_000, render_us=100)
    _open(s, 0)  # the first develop holds the develop lane
    first, _ = s.submit_export(0, 1, _edit(0.1), EXPORTS[:1])
    second, outs = s.submit_export(0, 2, _edit(0.2), EXPORTS[:1])
    res = {r["request_id"]: r for r in _results(s, 5000)}
    assert res[first]["status"] == RD_CANCELLED and res[second]["status"] == RD_OK
    assert np.all(outs[0] == 2)
    s.close()


def test_dry_export_is_admitted_against_the_budget():
    layers, develop = _footprint(1024, 1024, 512, 512)
    export = 32 * 1024 * 1024 + 6 * 1024 * 1024 + 64 * MB
    s = PreviewServer.dry(budget_bytes=layers + develop + MB, develop_us=1000, render_us=100)
    _open(s, 0)
    _results(s)
    assert export > develop + MB
    rid, _ = s.submit_export(0, 1, _edit(0.1), EXPORTS[1:])
    res = {r["request_id"]: r for r in _results(s)}
    assert res[rid]["status"] == RD_OVER_BUDGET  # the export's transient does not fit
    s.close()
    s = PreviewServer.dry(budget_bytes=layers + export + MB, develop_us=1000, render_us=100)
    _open(s, 0)
    _results(s)
    rid, _ = s.submit_export(0, 1, _edit(0.1), EXPORTS[1:])
    res = {r["request_id"]: r for r in _results(s)}
    assert res[rid]["status"] == RD_OK and s.stats()["peak_resident_bytes"] <= layers + export + MB
    s.close()


def test_dry_close_cancels_a_pending_export():
    s = PreviewServer.dry(develop_us=200_000, render_us=100)
    _open(s, 0)
    _open(s, 1)
    rid, _ = s.submit_export(1, 1, _edit(0.1), EXPORTS[:1])
    s.close_image(1)
    res = {r["request_id"]: r for r in _results(s, 5000)}
    assert res[rid]["status"] == RD_CANCELLED
    s.close()


def test_dry_export_files_fill_the_client_buffers():
    s = PreviewServer.dry(develop_us=1000, render_us=100)
    _open(s, 3)
    _results(s)
    specs = [OutputSpec(format="srgb8"), OutputSpec(format="srgb16"), OutputSpec(format="srgb8")]
    files = [{"format": "png"}, {"format": "png", "icc": b"profile"}, {"format": "jpeg", "quality": 80}]
    rid, outs, sizes = s.submit_export_files(3, 1, _edit(0.7), specs, files)
    res = {r["request_id"]: r for r in _results(s)}
    assert res[rid]["kind"] == EXPORT and res[rid]["status"] == RD_OK
    assert [int(n) for n in sizes] == [o.nbytes for o in outs]  # the dry executor fills whole buffers
    assert np.all(outs[2] == 7)
    s.close()


def test_export_files_are_validated_at_submission():
    from rohditor_gb300.processor import GpuPreviewError

    s = PreviewServer.dry(develop_us=1000, render_us=100)
    _open(s, 0)
    _results(s)
    bad = [
        ([OutputSpec(format="srgb16")], [{"format": "jpeg"}]),                        # JPEG takes 8-bit rows
        ([OutputSpec(format="extended_f16", headroom=2.0)], [{"format": "png"}]),  # PNG takes display rows
        ([OutputSpec(format="srgb8")], [{"format": "jpeg", "quality": 0}]),
        ([OutputSpec(format="srgb8")], [{"format": "jpeg", "quality": 101}]),
        ([OutputSpec(format="srgb8")], [{"format": "jpeg", "exif": bytes(65528)}]),  # more than one APP1
    ]
    for specs, files in bad:
        with pytest.raises(GpuPreviewError) as err:
            s.submit_export_files(0, 1, _edit(0.1), specs, files)
        assert err.value.code == 8
    s.close()


def test_dry_export_files_are_charged_their_encoder():
    # A file export holds the output rows, the file and the encoder's scratch:
    # a budget that admits the rows-only export refuses the same output as a PNG.
    layers, develop = _footprint(1024, 1024, 512, 512)
    rows_export = 32 * 1024 * 1024 + 3 * 1024 * 1024 + 64 * MB
    s = PreviewServer.dry(budget_bytes=layers + rows_export + MB, develop_us=1000, render_us=100)
    _open(s, 0)
    _results(s)
    rid, _ = s.submit_export(0, 1, _edit(0.1), [OutputSpec(format="srgb8")])
    assert {r["request_id"]: r for r in _results(s)}[rid]["status"] == RD_OK
    rid, _, _ = s.submit_export_files(0, 2, _edit(0.1), [OutputSpec(format="srgb8")], [{"format": "png"}])
    assert {r["request_id"]: r for r in _results(s)}[rid]["status"] == RD_OVER_BUDGET
    s.close()


@pytest.mark.gpu
def test_served_export_files_match_the_direct_encoders(device):
    """Served PNG and JPEG exports equal the encoders run on the direct path's
    output rows, byte for byte, metadata included."""
    from rohditor_gb300 import GpuSensorProcessor, GpuSpatialProcessor, GpuPreviewProcessor, JpegEncoder, PngEncoder
    from rohditor_gb300.workloads import CAMERA_TO_REC2020, sixteen_knot_curve

    server = PreviewServer(0, budget_bytes=2 << 30)
    raw, desc, cap, optics, wb = _image(w=640, h=480, seed=31)
    server.open(6, raw, desc, cap, optics, (320, 240), wb, CAMERA_TO_REC2020)
    color = ColorContract(wb_gains=wb, camera_to_rec2020=CAMERA_TO_REC2020, exposure_ev=0.2,
                          tone_lut=sixteen_knot_curve(seed=6))
    icc, exif = bytes(range(256)) * 3, b"II*\x00" + bytes(40)
    specs = [OutputSpec(format="srgb8"), OutputSpec(format="srgb16", dither="ordered8x8"),
             OutputSpec(format="srgb8", orientation="rotate90")]
    files = [{"format": "png", "icc": icc, "exif": exif}, {"format": "png"},
             {"format": "jpeg", "quality": 85, "icc": icc, "exif": exif}]
    rid, outs, sizes = server.submit_export_files(6, 1, color, specs, files)
    server.drain()
    res = {r["request_id"]: r for r in server.poll(64)}
    assert res[rid]["kind"] == EXPORT and res[rid]["status"] == RD_OK
    src = GpuSensorProcessor(device).develop(raw, desc, cap)
    base = GpuSpatialProcessor(device).reduce_preview(src, optics, (640, 480), wb, CAMERA_TO_REC2020)
    preview = GpuPreviewProcessor(device)
    for spec, f, out, n in zip(specs, files, outs, sizes):
        rows, _, _ = preview.render_output(base, color, spec)
        rows = rows.reshape(rows.shape[0], -1, 3)
        if f["format"] == "png":
            ref = PngEncoder(device).encode(rows, f.get("icc", b""), f.get("exif"))
        else:
            ref = JpegEncoder(device).encode(rows, f["quality"], f.get("icc", b""), f.get("exif"))
        assert out[:int(n)].tobytes() == ref, (spec.format, f["format"])
    base.release()
    src.release()
    server.close()


@pytest.mark.gpu
def test_served_export_matches_the_direct_path(device):
    """A served full-resolution export equals develop + spatial pass at the crop
    size + rd_render_output of the same settings, bit for bit."""
    from rohditor_gb300 import GpuPreviewProcessor, GpuSensorProcessor, GpuSpatialProcessor
    from rohditor_gb300.workloads import CAMERA_TO_REC2020, hsl_bands, sixteen_knot_curve

    server = PreviewServer(0, budget_bytes=2 << 30)
    raw, desc, cap, optics, wb = _image(w=768, h=512, seed=21)
    server.open(5, raw, desc, cap, optics, (384, 256), wb, CAMERA_TO_REC2020)
    color = ColorContract(wb_gains=wb, camera_to_rec2020=CAMERA_TO_REC2020, exposure_ev=0.3,
                          tone_lut=sixteen_knot_curve(seed=4), hsl=hsl_bands(seed=4))
    specs = EXPORTS + [OutputSpec(format="srgb16", dither="ordered8x8", orientation="rotate90")]
    rid, outs = server.submit_export(5, 1, color, specs)
    server.drain()
    res = {r["request_id"]: r for r in server.poll(64)}
    assert res[rid]["kind"] == EXPORT and res[rid]["status"] == RD_OK
    src = GpuSensorProcessor(device).develop(raw, desc, cap)
    base = GpuSpatialProcessor(device).reduce_preview(src, optics, (768, 512), wb, CAMERA_TO_REC2020)
    preview = GpuPreviewProcessor(device)
    for spec, out in zip(specs, outs):
        ref, _, _ = preview.render_output(base, color, spec)
        assert np.array_equal(out.view(np.uint8), ref.view(np.uint8)), spec.format
    base.release()
    src.release()
    st = server.stats()
    assert st["exports"] == 1 and st["peak_resident_bytes"] <= 2 << 30
    server.close()


@pytest.mark.gpu
def test_served_edits_match_the_render_entry_point(device):
    """Batched served renders of several images equal rd_render of the same bases."""
    from rohditor_gb300 import GpuPreviewProcessor, GpuSensorProcessor, GpuSpatialProcessor
    from rohditor_gb300.workloads import CAMERA_TO_REC2020, hsl_bands, sixteen_knot_curve
    from rohditor_gb300 import standard_base_lut

    server = PreviewServer(0)
    images = {}
    for i in range(3):
        raw, desc, cap, optics, wb = _image(w=640, h=480, seed=10 + i)
        target = (320, 240)
        server.open(i, raw, desc, cap, optics, target, wb, CAMERA_TO_REC2020)
        images[i] = (raw, desc, cap, optics, wb, target)
    server.drain()
    assert all(r["status"] == RD_OK for r in server.poll(64))
    colors = {i: ColorContract(wb_gains=images[i][4], camera_to_rec2020=CAMERA_TO_REC2020, exposure_ev=0.2 * i,
                               base_lut=standard_base_lut(), tone_lut=sixteen_knot_curve(seed=i), hsl=hsl_bands(seed=i))
              for i in range(3)}
    for i in range(3):
        server.submit_edit(i, 1, colors[i])
    server.drain()
    res = server.poll(64)
    assert sorted(r["image_id"] for r in res) == [0, 1, 2] and all(r["status"] == RD_OK for r in res)
    for i in range(3):
        raw, desc, cap, optics, wb, target = images[i]
        src = GpuSensorProcessor(device).develop(raw, desc, cap)
        base = GpuSpatialProcessor(device).reduce_preview(src, optics, target, wb, CAMERA_TO_REC2020)
        ref, hist = GpuPreviewProcessor(device).render(base, colors[i])
        out, served_hist, rev = server.read_output(i)
        assert rev == 1
        assert np.array_equal(out, ref)
        assert np.array_equal(served_hist[:256], hist.red) and np.array_equal(served_hist[768:], hist.luminance)
        base.release()
        src.release()
    server.close()


@pytest.mark.gpu
def test_edits_overlapping_a_develop_equal_their_solo_renders(device):
    """Continuous batching: edits of three images submitted while a large
    develop of a fourth image runs on the develop lane render on the render
    lane meanwhile (they finish before the develop does), and every result is
    the same as alone: each edited image's output equals rd_render of its base
    with its last settings, and the developed image's re-render equals a solo
    develop + spatial pass + render with the new capture settings
    (the newest-wins mailbox of crates/engine/src/coordinator/scheduler.rs:44-166)."""
    from rohditor_gb300 import GpuPreviewProcessor, GpuSensorProcessor, GpuSpatialProcessor, standard_base_lut
    from rohditor_gb300.workloads import CAMERA_TO_REC2020, hsl_bands, sixteen_knot_curve

    server = PreviewServer(0)
    images = {}
    for i in range(3):
        raw, desc, cap, optics, wb = _image(w=640, h=480, seed=30 + i)
        images[i] = (raw, desc, cap, optics, wb, (320, 240))
    big = 3
    raw, desc, cap, optics, wb = _image(w=8256, h=5504, seed=40)
    images[big] = (raw, desc, cap, optics, wb, (2560, 1707))
    for i, (raw, desc, cap, optics, wb, target) in images.items():
        server.open(i, raw, desc, cap, optics, target, wb, CAMERA_TO_REC2020)
    server.drain(120000)
    assert all(r["status"] == RD_OK for r in server.poll(64))

    def colour(i, k):
        return ColorContract(wb_gains=images[i][4], camera_to_rec2020=CAMERA_TO_REC2020, exposure_ev=0.1 * k - 0.2,
                             base_lut=standard_base_lut(), tone_lut=sixteen_knot_curve(seed=7 * i + k),
                             hsl=hsl_bands(seed=11 * i + k))

    big_colour = colour(big, 0)
    server.submit_edit(big, 1, big_colour)
    server.drain(60000)
    server.poll(64)
    new_cap = CaptureContract(amount=0.8, radius=0.9, noise_protection=0.3, ceilings=images[big][2].ceilings,
                              iterations=20)
    submitted = {}
    t0 = time.perf_counter()
    dev_id = server.submit_develop(big, 2, new_cap, images[big][3])
    submitted[dev_id] = 0.0
    last = {}
    for k in range(1, 4):
        for i in range(3):
            rid = server.submit_edit(i, 1 + k, colour(i, k))
            submitted[rid] = 1e3 * (time.perf_counter() - t0)
            last[i] = (rid, k)
        time.sleep(0.002)
    server.drain(120000)
    res = {r["request_id"]: r for r in server.poll(256)}
    develop = res[dev_id]
    assert develop["kind"] == DEVELOP and develop["status"] == RD_OK
    develop_done = develop["latency_ms"]
    overlapped = [rid for rid, r in res.items()
                  if r["kind"] == EDIT and r["status"] == RD_OK and submitted[rid] + r["latency_ms"] < develop_done]
    assert overlapped, "no edit finished while the develop was running"

    preview = GpuPreviewProcessor(device)
    for i in range(3):
        raw, desc, cap, optics, wb, target = images[i]
        rid, k = last[i]
        assert res[rid]["status"] == RD_OK
        src = GpuSensorProcessor(device).develop(raw, desc, cap)
        base = GpuSpatialProcessor(device).reduce_preview(src, optics, target, wb, CAMERA_TO_REC2020)
        ref, hist = preview.render(base, colour(i, k))
        out, served_hist, rev = server.read_output(i)
        assert rev == 1 + k
        assert np.array_equal(out, ref)
        assert np.array_equal(served_hist[:256], hist.red) and np.array_equal(served_hist[768:], hist.luminance)
        base.release()
        src.release()
    raw, desc, cap, optics, wb, target = images[big]
    src = GpuSensorProcessor(device).develop(raw, desc, new_cap)
    base = GpuSpatialProcessor(device).reduce_preview(src, optics, target, wb, CAMERA_TO_REC2020)
    ref, _ = preview.render(base, big_colour)
    out, _, _ = server.read_output(big)
    assert np.array_equal(out, ref)
    base.release()
    src.release()
    server.close()

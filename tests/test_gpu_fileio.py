"""Files on device-resident data: .pj / .if streamed straight to and from
device memory, pj2if's transpose and if2's comparative statistics, checked
against files and numbers the reference itself wrote (tests/golden/io.npz,
made by tests/golden/make_golden.py) and against the FP64 oracle.

Bars: file bytes and pixel values bit-exact; e of comparativeStatistics
exact; d and r within 1e-12 relative of the reference's sequential FP64 sums
(the device sums in a different, fixed order)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

IO_SCANS = ["herman_eql", "shepp_eqa_even", "pulse_par"]
REL = 1e-12


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ctsim_gb300 as cg
    from ctsim_gb300 import device, fileio
    return torch, cg, device, fileio


def golden_pj(golden, tmp_path, name):
    path = tmp_path / (name + ".pj")
    path.write_bytes(golden("io")[name + "/pj"].tobytes())
    return path


def to_device(torch, device, data, angles):
    nv, nd = data.shape
    sino = torch.zeros((nv, device.pitch_for(nd)), dtype=torch.float32, device="cuda")
    sino[:, :nd] = torch.from_numpy(np.ascontiguousarray(data)).cuda()
    ang = torch.from_numpy(np.ascontiguousarray(angles, np.float64)).cuda()
    return sino, ang


@pytest.mark.parametrize("name", IO_SCANS)
def test_pj_read_device_matches_reference_file(gpu, golden, tmp_path, name):
    torch, cg, device, fileio = gpu
    path = golden_pj(golden, tmp_path, name)
    ref = fileio.read_pj(path)
    info, remark, sino, ang, n = device.read_pj(path)
    g = info.geometry
    assert n == ref.nView == g.n_view and g.n_det == ref.nDet and g.geometry == ref.geometry
    assert (g.rot_start, g.rot_inc, g.det_start, g.det_inc, g.view_diameter, g.focal_length,
            g.source_detector_length, g.fan_beam_angle) == \
        (ref.rotStart, ref.rotInc, ref.detStart, ref.detInc, ref.viewDiameter, ref.focalLength,
         ref.sourceDetectorLength, ref.fanBeamAngle)
    assert info.calc_time == ref.calcTime and tuple(info.date) == tuple(ref.date)
    assert remark == ref.remark
    s = sino.cpu().numpy()
    np.testing.assert_array_equal(s[:, :ref.nDet], ref.data)
    assert not s[:, ref.nDet:].any()   # pad columns zeroed
    np.testing.assert_array_equal(ang.cpu().numpy(), ref.angles)


@pytest.mark.parametrize("name", IO_SCANS)
def test_pj_write_device_is_byte_identical(gpu, golden, tmp_path, name):
    torch, cg, device, fileio = gpu
    path = golden_pj(golden, tmp_path, name)
    ref = fileio.read_pj(path)
    info, remark = device.read_pj_header(path)
    sino, ang = to_device(torch, device, ref.data, ref.angles)
    out = tmp_path / "out.pj"
    device.write_pj(out, info, remark, sino, ang)
    assert out.read_bytes() == path.read_bytes()


@pytest.mark.parametrize("name", IO_SCANS)
def test_pj_pack_unpack_records(gpu, golden, tmp_path, name):
    """The device-to-device record calls: pack gives the file's bytes after the
    header; unpack inverts it and flags a record with a wrong detector count."""
    torch, cg, device, fileio = gpu
    path = golden_pj(golden, tmp_path, name)
    ref = fileio.read_pj(path)
    info, _ = device.read_pj_header(path)
    sino, ang = to_device(torch, device, ref.data, ref.angles)
    rec = device.pj_pack(sino, ref.nDet, ang)
    assert rec.cpu().numpy().tobytes() == path.read_bytes()[info.header_size:]
    s2, a2, bad, first = device.pj_unpack(rec, ref.nView, ref.nDet)
    assert bad == 0 and torch.equal(s2, sino) and torch.equal(a2, ang)
    # records at a 4-byte (not 16-byte) aligned address take the word-by-word path
    big = torch.zeros(rec.numel() + 1, dtype=torch.int32, device="cuda")
    device.pj_pack(sino, ref.nDet, ang, out=big[1:])
    assert torch.equal(big[1:], rec)
    s3, a3, bad, _ = device.pj_unpack(big[1:], ref.nView, ref.nDet)
    assert bad == 0 and torch.equal(s3, sino) and torch.equal(a3, ang)
    rec[(3 + ref.nDet) * 4 + 2] = ref.nDet - 1   # view 4's detector count
    rec[(3 + ref.nDet) * 6 + 2] = 0              # and view 6's
    _, _, bad, first = device.pj_unpack(rec, ref.nView, ref.nDet)
    assert (bad, first) == (2, 4)


def test_pj_round_trip_many_chunks(gpu, tmp_path):
    """9216 views x 1024 detectors (38 MB, five 8 MiB chunks each way): the
    device writer's file equals the host restatement's, and reads back exact."""
    torch, cg, device, fileio = gpu
    rng = np.random.default_rng(5)
    nv, nd = 9216, 1024
    data = rng.standard_normal((nv, nd)).astype(np.float32)
    angles = np.cumsum(rng.random(nv)) * 1e-3
    pj = fileio.ProjectionFile(nv, nd, 2, 1.5, 0.1, 2 * np.pi / 1152, -0.7, 0.0013, 2.1, 3.3,
                               6.6, 0.8, date=(2026, 1, 2, 3, 4, 5), remark="round trip",
                               angles=angles, data=data)
    host = tmp_path / "host.pj"
    fileio.write_pj(host, pj)
    info, remark = device.read_pj_header(host)
    sino, ang = to_device(torch, device, data, angles)
    dev = tmp_path / "dev.pj"
    device.write_pj(dev, info, remark, sino, ang)
    assert dev.read_bytes() == host.read_bytes()
    info2, remark2, sino2, ang2, n = device.read_pj(dev)
    assert n == nv and remark2 == "round trip"
    assert torch.equal(sino2, sino) and torch.equal(ang2, ang)


def test_pj_short_file_and_bad_record(gpu, golden, tmp_path):
    torch, cg, device, fileio = gpu
    path = golden_pj(golden, tmp_path, "herman_eql")
    ref = fileio.read_pj(path)
    raw = path.read_bytes()
    info, _ = device.read_pj_header(path)
    rec = 12 + 4 * ref.nDet
    # ends inside view 37: views 0..36 kept (projections.cpp:650-655), the rest zero
    cut = tmp_path / "cut.pj"
    cut.write_bytes(raw[:info.header_size + 37 * rec + 100])
    _, _, sino, ang, n = device.read_pj(cut)
    assert n == 37
    s = sino.cpu().numpy()
    np.testing.assert_array_equal(s[:37, :ref.nDet], ref.data[:37])
    assert not s[37:].any() and not ang.cpu().numpy()[37:].any()
    # view 5 claims a different detector count
    bad = bytearray(raw)
    off = info.header_size + 5 * rec + 8
    bad[off:off + 4] = (ref.nDet + 1).to_bytes(4, "little")
    badp = tmp_path / "bad.pj"
    badp.write_bytes(bytes(bad))
    with pytest.raises(cg.CtgpuError) as ei:
        device.read_pj(badp)
    assert ei.value.code == 6 and "first at view 5" in str(ei.value)
    with pytest.raises(cg.CtgpuError):
        device.read_pj(tmp_path / "missing.pj")


@pytest.mark.parametrize("name", IO_SCANS)
def test_pj2if_matches_reference(gpu, golden, tmp_path, name):
    torch, cg, device, fileio = gpu
    path = golden_pj(golden, tmp_path, name)
    info, _, sino, _, _ = device.read_pj(path)
    im = device.sino_to_image(sino, info.geometry.n_det)
    np.testing.assert_array_equal(im.cpu().numpy(), golden("io")[name + "/pj2if"])


def test_sino_to_image_ragged_sizes(gpu):
    torch, cg, device, fileio = gpu
    rng = np.random.default_rng(9)
    for nv, nd in ((1, 1), (33, 31), (1000, 733), (64, 2048)):
        data = rng.standard_normal((nv, nd)).astype(np.float32)
        sino, _ = to_device(torch, device, data, np.zeros(nv))
        im = device.sino_to_image(sino, nd).cpu().numpy()
        np.testing.assert_array_equal(im, data[::-1].T)


def test_if_device_write_read(gpu, tmp_path):
    torch, cg, device, fileio = gpu
    rng = np.random.default_rng(3)
    a = torch.from_numpy(rng.standard_normal((1500, 1111)).astype(np.float32)).cuda()
    info = cg._lib.IfInfo()
    info.increment_known, info.extent_known = 1, 1
    info.increment[:] = [0.01, 0.02]
    info.extent[:] = [-1.0, 1.0, -2.0, 2.0]
    info.scale_pv = 1.0
    labels = [(1, "first label", 1.25, (2025, 7, 8, 9, 10, 11)), (2, "", 0.0, (1, 1, 1, 0, 0, 0))]
    f = tmp_path / "a.if"
    device.write_if(f, a, info, labels)
    h = fileio.read_if(f)
    assert (h.nx, h.ny, h.pixel_format, h.pixel_size, h.data_type) == (1500, 1111, 7, 4, 1)
    assert h.increment == (0.01, 0.02) and h.extent == (-1.0, 1.0, -2.0, 2.0)
    assert h.increment_known == 1 and h.extent_known == 1 and h.scalePV == 1.0
    np.testing.assert_array_equal(h.data, a.cpu().numpy())
    assert [(l[0], l[1], l[2], l[3]) for l in h.labels] == [(1, "first label", 1.25,
                                                            (2025, 7, 8, 9, 10, 11)),
                                                           (2, "", 0.0, (1, 1, 1, 0, 0, 0))]
    assert device.read_if_labels(f) == h.labels
    _, b = device.read_if(f)
    assert torch.equal(a, b)
    # FP64 pixels are converted on the device
    d64 = rng.standard_normal((70, 45))
    f64 = tmp_path / "b.if"
    fileio.write_if(f64, fileio.ImageFileData(70, 45, 8, 8, 1, data=d64))
    hi, c = device.read_if(f64)
    assert hi.pixel_size == 8
    np.testing.assert_array_equal(c.cpu().numpy(), d64.astype(np.float32))


@pytest.mark.parametrize("k", range(5))
def test_image_compare_matches_reference(gpu, golden, oracle, k):
    torch, cg, device, fileio = gpu
    g = golden("io")
    a, b, dre = g["comp/%d/a" % k], g["comp/%d/b" % k], g["comp/%d/dre" % k]
    d, r, e = device.image_compare(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda())
    assert e == dre[2]
    for got, want in ((d, dre[0]), (r, dre[1])):
        assert abs(got - want) <= REL * abs(want), (k, got, want)
    # the oracle restatement is the reference's loop: identical numbers
    assert oracle.image_compare(a, b) == tuple(dre)


def test_image_compare_batched_against_oracle(gpu, oracle):
    """eight 512 x 512 pairs in one call; odd sizes; degenerate images."""
    torch, cg, device, fileio = gpu
    rng = np.random.default_rng(21)
    a = (rng.standard_normal((8, 512, 512)) * 2 + 0.3).astype(np.float32)
    b = (a + 0.05 * rng.standard_normal(a.shape)).astype(np.float32)
    got = device.image_compare(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda())
    dev = device.image_compare_device(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda())
    np.testing.assert_array_equal(dev.cpu().numpy(), got)   # same kernels, same order
    # an odd-sized batch: unaligned second image, word-by-word loads
    x = torch.from_numpy(a[:3, :511, :511].copy()).cuda()
    y = torch.from_numpy(b[:3, :511, :511].copy()).cuda()
    g3 = device.image_compare(x, y)
    for i in range(3):
        want = oracle.image_compare(a[i, :511, :511], b[i, :511, :511])
        assert g3[i, 2] == want[2]
        np.testing.assert_allclose(g3[i, :2], want[:2], rtol=REL, atol=0)
    for i in range(8):
        want = oracle.image_compare(a[i], b[i])
        assert got[i, 2] == want[2]
        np.testing.assert_allclose(got[i, :2], want[:2], rtol=REL, atol=0)
    for nx, ny in ((1, 7), (7, 1), (3, 5), (513, 257)):
        x = rng.standard_normal((nx, ny)).astype(np.float32)
        y = rng.standard_normal((nx, ny)).astype(np.float32)
        d, r, e = device.image_compare(torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda())
        want = oracle.image_compare(x, y)
        assert e == want[2] and (e == -1.0) == (nx < 2 or ny < 2)
        np.testing.assert_allclose((d, r), want[:2], rtol=REL, atol=0)
    # constant first image: sum (a - mean)^2 = 0, d = inf as in the reference
    x = np.full((16, 16), 0.5, np.float32)
    y = rng.standard_normal((16, 16)).astype(np.float32)
    d, r, e = device.image_compare(torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda())
    want = oracle.image_compare(x, y)
    assert np.isinf(d) and np.isinf(want[0]) and e == want[2]


def test_image_arith(gpu):
    torch, cg, device, fileio = gpu
    rng = np.random.default_rng(4)
    a = rng.standard_normal((301, 77)).astype(np.float32)
    b = rng.standard_normal((301, 77)).astype(np.float32)
    b[0, :5] = 0.0
    a[0, 0] = 0.0
    ta, tb = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    with np.errstate(divide="ignore", invalid="ignore"):
        for op, want in (("add", a + b), ("subtract", a - b), ("multiply", a * b),
                         ("divide", a / b)):
            np.testing.assert_array_equal(device.image_arith(op, ta, tb).cpu().numpy(), want)
    with pytest.raises(cg.CtgpuError):
        device.image_arith("modulo", ta, tb)

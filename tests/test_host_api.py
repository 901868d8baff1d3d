"""Host-side behaviour of the drop-in API that needs no GPU: the class
family, constructor parsing, argument validation with the reference's
exception classes and messages, zeros(), Ranges containers, thread-interval
flattening and the quaternion helpers."""
import numpy as np
import pytest

import so3g_gb300
from so3g_gb300 import RangesInt32, RangesMatrix
from so3g_gb300.projeng import derive_ranges, flatten_ranges, _edges_to_ranges
from so3g_gb300.proj import quat

DEG = np.pi / 180


def test_class_family():
    names = set(so3g_gb300.ENGINES)
    # 8 coordinate systems x 3 spins x 2 tilings x 2 interpolations, 6
    # HEALPix classes and 2 Precomp classes (src/Projection.cxx:2337-2358).
    assert len(names) == 8 * 3 * 2 * 2 + 6 + 2
    for n in ["ProjEng_CAR_TQU_NonTiled", "ProjEng_ZEA_QU_Tiled_Bilinear",
              "ProjEng_HP_T_Tiled", "ProjEng_Precomp_NonTiled", "ProjEng_Flat_T_NonTiled"]:
        assert hasattr(so3g_gb300, n)
    e = so3g_gb300.ProjEng_TAN_QU_Tiled((10, 20, 1e-3, 1e-3, 5., 10., 4, 6))
    assert e.index_count == 3 and e.comp_count == 2
    assert so3g_gb300.ProjEng_HP_TQU_NonTiled((16, 1, None, None)).index_count == 1
    assert so3g_gb300.ProjEng_HP_T_Tiled((16, 1, 4, None)).index_count == 2


def test_constructor_errors():
    with pytest.raises(ValueError, match="Invalid nside 12"):
        so3g_gb300.ProjEng_HP_T_NonTiled((12, 1, None, None))
    with pytest.raises(ValueError, match="RING not supported for tiled maps"):
        so3g_gb300.ProjEng_HP_T_Tiled((16, 0, 4, None))
    with pytest.raises(ValueError, match="Invalid nside_tile 32 > nside 16"):
        so3g_gb300.ProjEng_HP_T_Tiled((16, 1, 32, None))


def test_zeros():
    e = so3g_gb300.ProjEng_CAR_TQU_NonTiled((10, 20, 1e-3, 1e-3, 5., 10.))
    assert e.zeros(3).shape == (3, 10, 20)
    assert e.zeros((3, 3)).shape == (3, 3, 10, 20)
    assert e.zeros("x") is None
    t = so3g_gb300.ProjEng_CAR_T_Tiled((10, 20, 1e-3, 1e-3, 5., 10., 4, 6, [0, 4, 11]))
    z = t.zeros(1)
    assert len(z) == 3 * 4
    assert [i for i, x in enumerate(z) if x is not None] == [0, 4, 11]
    assert z[11].shape == (1, 2, 2)          # edge tile cropped to the map
    nt = so3g_gb300.ProjEng_CAR_T_Tiled((10, 20, 1e-3, 1e-3, 5., 10., 4, 6))
    with pytest.raises(RuntimeError, match="Cannot create blank tiled map"):
        nt.zeros(1)
    hp = so3g_gb300.ProjEng_HP_T_Tiled((16, 1, 4, [1, 2]))
    z = hp.zeros(2)
    assert z[1].shape == (2, 16) and z[0] is None


def _args(n_det=3, n_time=50):
    bore = np.zeros((n_time, 4))
    bore[:, 0] = 1
    dets = np.zeros((n_det, 4))
    dets[:, 0] = 1
    resp = np.ones((n_det, 2), np.float32)
    sig = np.ones((n_det, n_time), np.float32)
    return bore, dets, resp, sig


def test_validation_errors_precede_device_work():
    """All of these are raised on the host before any GPU call."""
    e = so3g_gb300.ProjEng_CAR_TQU_NonTiled((10, 20, 1e-3, 1e-3, 5., 10.))
    bore, dets, resp, sig = _args()
    with pytest.raises(TypeError, match="Argument 'boresight' does not expose buffer"):
        e.to_map(None, 7, dets, resp, sig)
    with pytest.raises(ValueError, match="Expected buffer 'boresight' to contain items of "
                                         "type float64."):
        e.to_map(None, bore.astype(np.float32), dets, resp, sig)
    with pytest.raises(RuntimeError, match=r"Buffer 'detectors' has incompatible shape: "
                                           r"Expected \(\*, 4\) but got \(3, 3\)."):
        e.to_map(None, bore, dets[:, :3], resp, sig)
    d = dets.copy()
    d[2, 1] = np.nan
    with pytest.raises(ValueError, match=r"Pointing offset error: nan found at index 2."):
        e.to_map(None, bore, d, resp, sig)
    # The reference's own check (component axis; its message), then the
    # pixel axes, which the reference leaves unchecked.
    with pytest.raises(RuntimeError, match=r"Buffer 'map' has incompatible shape: "
                                           r"Expected \(3, \*, \*\) but got \(1, 10, 20\)\.\."):
        e.to_map(np.zeros((1, 10, 20)), bore, dets, resp, sig)
    with pytest.raises(RuntimeError, match=r"Buffer 'map' has incompatible shape: "
                                           r"Expected \(3, 10, 20\) but got \(3, 10, 21\)\.\."):
        e.to_map(np.zeros((3, 10, 21)), bore, dets, resp, sig)
    with pytest.raises(RuntimeError, match="must contain \\(n_det\\) vectors"):
        e.to_map(None, bore, dets, resp, sig[:2])
    with pytest.raises(RuntimeError, match=r"Buffer 'signal' has incompatible shape"):
        e.to_map(None, bore, dets, resp, sig[:, :10])
    with pytest.raises(ValueError, match="'det_weights' to contain items of type float32"):
        e.to_map(None, bore, dets, resp, sig, np.ones(3))
    with pytest.raises(RuntimeError, match=r"Buffer 'response' has incompatible shape"):
        e.to_map(None, bore, dets, resp[:2], sig)
    with pytest.raises(RuntimeError, match=r"Buffer 'map' has incompatible shape"):
        e.to_weight_map(np.zeros((3, 10, 20)), bore, dets, resp)
    with pytest.raises(RuntimeError, match="No tiles in this pixelization."):
        e.tile_hits(bore, dets)
    # Signal as a list of per-detector rows is validated per row.
    with pytest.raises(RuntimeError, match="signal"):
        e.to_map(None, bore, dets, resp, [sig[0], sig[1], sig[2][:10]])


def test_tiled_map_validation():
    t = so3g_gb300.ProjEng_CAR_T_Tiled((10, 20, 1e-3, 1e-3, 5., 10., 4, 6, [0, 1]))
    bore, dets, resp, sig = _args()
    m = t.zeros(1)
    m[1] = None
    with pytest.raises(RuntimeError, match=r"Tiling problem \(index 1\): Projector expects "
                                           r"tile but it is missing."):
        t.to_map(m, bore, dets, resp, sig)
    with pytest.raises(RuntimeError, match="Expected a list of 12 tiles"):
        t.to_map(m[:5], bore, dets, resp, sig)
    m = t.zeros(1)
    m[0] = np.zeros((1, 4, 5))
    with pytest.raises(RuntimeError, match=r"Expected \(1, 4, 6\) but got \(1, 4, 5\)"):
        t.to_map(m, bore, dets, resp, sig)


def test_ranges():
    r = RangesInt32(100)
    r.add_interval(10, 20).add_interval(15, 30).add_interval(50, 60)
    assert r.ranges().tolist() == [[10, 30], [50, 60]]
    assert r.mask().sum() == 30
    c = ~r
    assert c.ranges().tolist() == [[0, 10], [30, 50], [60, 100]]
    r2 = RangesInt32.from_mask(r.mask())
    assert r2.ranges().tolist() == r.ranges().tolist()
    a = RangesInt32(100).add_interval(0, 40)
    assert (a * r).ranges().tolist() == [[10, 30]]
    assert (a + r).ranges().tolist() == [[0, 40], [50, 60]]
    n = RangesInt32(10).append_interval_no_check(2, 5).append_interval_no_check(5, 7)
    assert n.ranges().tolist() == [[2, 5], [5, 7]]      # not merged
    rm = RangesMatrix([RangesInt32(10), n])
    assert rm.shape == (2, 10)
    assert rm.mask().sum() == 5
    rm3 = RangesMatrix([rm, rm])
    assert rm3.shape == (2, 2, 10)
    assert rm3[1, 1].ranges().tolist() == [[2, 5], [5, 7]]


def test_derive_ranges_forms():
    n_det, n_time = 2, 10

    def rm():
        return RangesMatrix([RangesInt32(n_time).add_interval(d, d + 3) for d in range(n_det)])

    assert derive_ranges(None, n_det, n_time) is None
    b = derive_ranges(rm(), n_det, n_time)
    assert len(b) == 1 and len(b[0]) == 1
    b = derive_ranges(RangesMatrix([rm(), rm(), rm()]), n_det, n_time)
    assert len(b) == 1 and len(b[0]) == 3
    b = derive_ranges([RangesMatrix([rm(), rm()]), RangesMatrix([rm()])], n_det, n_time)
    assert [len(x) for x in b] == [2, 1]
    seg, toff, boff = flatten_ranges(b)
    assert seg.shape == (6, 3)
    assert toff.tolist() == [0, 2, 4, 6] and boff.tolist() == [0, 2, 3]
    assert seg[:2].tolist() == [[0, 0, 3], [1, 1, 4]]
    with pytest.raises(RuntimeError, match="Expected RangesMatrix with n_det=3"):
        derive_ranges(rm(), 3, n_time)
    with pytest.raises(RuntimeError, match="Expected RangesMatrix with n_time=11"):
        derive_ranges(rm(), n_det, 11)


def test_edges_to_ranges():
    # det 0: labels 0 0 1 1 -1 -1 3 3 (n_domain 3 -> serial), det 1: all 2.
    e = np.array([[0, 0, 0], [0, 2, 1], [0, 4, -1], [0, 6, 3], [1, 0, 2]], np.int32)
    par, ser = _edges_to_ranges(e[::-1].copy(), 2, 8, 3)
    assert par[0][0].ranges().tolist() == [[0, 2]]
    assert par[1][0].ranges().tolist() == [[2, 4]]
    assert ser[0][0].ranges().tolist() == [[6, 8]]
    assert par[2][1].ranges().tolist() == [[0, 8]]


def test_quaternions():
    q = quat.euler(2, 0.3)
    assert isinstance(q, quat.quat)
    v = quat.euler(1, np.array([0.1, 0.2]))
    assert isinstance(v, quat.G3VectorQuat) and v.shape == (2, 4)
    p = q * v
    assert isinstance(p, quat.G3VectorQuat)
    # Rotations compose: euler(2, a) * euler(2, b) == euler(2, a + b).
    np.testing.assert_allclose(np.asarray(quat.euler(2, 0.3) * quat.euler(2, 0.4)),
                               np.asarray(quat.euler(2, 0.7)), atol=1e-15)
    lon, lat, psi = 0.4, -0.2, 0.1
    back = quat.decompose_lonlat(quat.rotation_lonlat(lon, lat, psi))
    np.testing.assert_allclose(back, (lon, lat, psi), atol=1e-12)
    xi, eta, gamma = 0.01, -0.02, 0.3
    np.testing.assert_allclose(quat.decompose_xieta(quat.rotation_xieta(xi, eta, gamma)),
                               (xi, eta, gamma), atol=1e-12)
    vq = quat.G3VectorQuat(np.tile([1., 0, 0, 0], (3, 1)))
    vq[1] = vq[1] * np.nan
    assert np.isnan(np.asarray(vq)[1]).all()


def test_projectionist_args():
    from so3g_gb300.proj import Projectionist, ProjectionistHealpix, SimpleWCS
    w = SimpleWCS("CAR", (10., 20.), (-0.5, 0.5), (50.5, 30.5))
    p = Projectionist.for_geom((60, 100), w)
    assert p.proj_name == "CAR"
    args = p._get_pixelizor_args()
    assert args[:2] == (60, 100)
    np.testing.assert_allclose(args[2:4], (0.5 * DEG, -0.5 * DEG))
    assert args[4:] == (30.5, 50.5)
    assert p.get_ProjEng("TQU").__class__.__name__ == "ProjEng_CAR_TQU_NonTiled"
    assert p.get_ProjEng("T", interpol="bilinear").__class__.__name__ == \
        "ProjEng_CAR_T_NonTiled_Bilinear"
    pt = Projectionist.for_tiled((60, 100), w, (20, 30))
    assert pt._get_pixelizor_args()[6:8] == (20, 30)
    assert len(pt.active_tiles) == 3 * 4
    hp = ProjectionistHealpix.for_healpix(64, nside_tile=4)
    assert hp._get_pixelizor_args() == (64, 1, 4, None)
    with pytest.raises(NotImplementedError):
        ProjectionistHealpix.for_healpix(64, nside_tile=4, ordering="RING")
    with pytest.raises(ValueError, match="Provide an output map"):
        p.to_map(None, None)


def test_install_as_so3g():
    import sys
    mod = so3g_gb300.install_as_so3g()
    assert sys.modules["so3g"] is mod
    import so3g
    assert so3g.ProjEng_CAR_TQU_NonTiled is so3g_gb300.ProjEng_CAR_TQU_NonTiled
    assert so3g.useful_info()["omp_num_threads"] >= 1


def test_host_signal_policy(monkeypatch):
    from so3g_gb300 import projeng
    monkeypatch.delenv("SO3G_GB300_HOST_SIGNAL", raising=False)
    assert projeng.host_signal_policy() == "auto"
    for name in ("auto", "direct", "mapped", "stream"):
        monkeypatch.setenv("SO3G_GB300_HOST_SIGNAL", name)
        assert projeng.host_signal_policy() == name
    monkeypatch.setenv("SO3G_GB300_HOST_SIGNAL", "bogus")
    with pytest.raises(ValueError, match="SO3G_GB300_HOST_SIGNAL"):
        projeng.host_signal_policy()


def test_detector_nan_check_remembers_clean_tensors():
    """A detector tensor found free of NaN is not checked again while it is
    the same tensor and unmodified; an in-place write brings the check
    back."""
    import torch
    from so3g_gb300 import projeng
    eng = so3g_gb300.ProjEng_CAR_TQU_NonTiled((10, 10, 1., 1., 5., 5.))
    bore = torch.zeros((7, 4), dtype=torch.float64)
    dets = torch.zeros((3, 4), dtype=torch.float64)
    dets[:, 0] = 1.
    eng._pointer(bore, dets)
    assert projeng._nan_checked(dets)
    eng._pointer(bore, dets)
    dets[1, 2] = float("nan")
    assert not projeng._nan_checked(dets)
    with pytest.raises(ValueError, match="nan found at index 1"):
        eng._pointer(bore, dets)
    other = dets.clone()
    assert not projeng._nan_checked(other)


def test_device_ranges_to_host():
    """DeviceRangesMatrix.to_host rebuilds the RangesMatrix from segments."""
    import torch
    from so3g_gb300.ranges import DeviceRangesMatrix
    seg = torch.tensor([[0, 2, 5], [0, 7, 9], [2, 0, 10]], dtype=torch.int32)
    d = DeviceRangesMatrix(seg, 3, 10, 10)
    assert d.shape == (3, 10) and len(d) == 3 and d.n_seg == 3
    m = d.mask()
    want = np.zeros((3, 10), bool)
    want[0, 2:5] = want[0, 7:9] = want[2, :] = True
    assert np.array_equal(m, want)
    assert np.array_equal(RangesMatrix.from_mask(want).mask(), want)

"""Host-side parts of the library and its Python mirror on the CPU: the
mirror's argument checks (the C ABI cannot know the length of a host array,
so shapes are checked before any call reaches the library; a recording
stand-in replaces the library in the tests that take the `lib` fixture) and
the host-only Manning class helper (the real library)."""
import numpy as np
import pytest

from sw2d_efdc_gb300 import api


class _Recorder:
    def __init__(self):
        self.calls = []

    def __getattr__(self, name):
        def f(*args):
            self.calls.append(name)
            return 0
        return f


@pytest.fixture
def lib(monkeypatch):
    rec = _Recorder()
    monkeypatch.setattr(api, "load", lambda *a: rec)
    return rec


def _model(R=6, C=5):
    m = object.__new__(api.Model)
    m._h = api.C.c_void_p(0)
    m.rows, m.cols, m._nfaces = R, C, 0
    return m


def test_point_sources_need_one_column_per_source(lib):
    m = _model()
    m.set_point_sources([3, 7], np.zeros((4, 2)), 60.0)
    m.set_point_sources([], np.zeros((0,)), 60.0)
    assert lib.calls == ["sw2d_set_point_sources"] * 2
    for q in (np.zeros(4), np.zeros((4, 3)), np.zeros((0, 2))):
        with pytest.raises(ValueError):
            m.set_point_sources([3, 7], q, 60.0)
    assert len(lib.calls) == 2


def test_grids_must_match_the_raster(lib):
    m = _model()
    m.set_dem(np.zeros((6, 5)))
    for f in (m.set_dem, m.set_depth, m.set_rain_field, m.set_coupling_mask):
        with pytest.raises(ValueError):
            f(np.zeros((5, 6)))
    with pytest.raises(ValueError):
        m.set_manning_classes(np.zeros((6, 4), np.uint8), [0.03])
    assert lib.calls == ["sw2d_set_dem"]


def test_coupling_calls_before_a_mask_have_no_faces(lib):
    m = _model()
    assert len(m.couple_sample()) == 0
    assert all(len(a) == 0 for a in m.coupling_faces())


def test_batch_submit_checks_every_grid_against_the_dem(lib):
    b = object.__new__(api.Batch)
    b._h = api.C.c_void_p(0)
    b._shapes = {}
    dem = np.zeros((8, 9))
    b.submit(dem, depth=np.zeros((8, 9)), manning_classes=np.zeros((8, 9), np.uint8), manning_table=[0.03],
             rain_weight=np.ones((8, 9), np.float32), rain_mm=[1.0, 2.0])
    assert lib.calls == ["sw2d_batch_submit"]
    bad = [dict(depth=np.zeros((9, 8))), dict(manning_classes=np.zeros((8, 8), np.uint8), manning_table=[0.03]),
           dict(rain_weight=np.ones(72, np.float32))]
    for kw in bad:
        with pytest.raises(ValueError):
            b.submit(dem, **kw)
    with pytest.raises(ValueError):
        b.submit(np.zeros(72))
    assert lib.calls == ["sw2d_batch_submit"]


def test_manning_classes_of_matches_numpy_unique():
    rng = np.random.default_rng(3)
    for shape, k in (((40, 30), 3), ((7, 11), 256), ((1, 1), 1), ((64, 64), 64)):
        values = np.sort(rng.uniform(0.01, 0.2, k))
        field = rng.choice(values, size=shape)
        cls, table = api.manning_classes_of(field)
        ref_table, ref_cls = np.unique(field, return_inverse=True)
        assert np.array_equal(table, ref_table)
        assert np.array_equal(cls, ref_cls.reshape(shape).astype(np.uint8))
        assert np.array_equal(table[cls], field)  # the round trip is exact


def test_manning_classes_of_refuses_what_a_table_cannot_hold():
    field = np.linspace(0.01, 0.2, 300)
    with pytest.raises(api.Sw2dError) as e:
        api.manning_classes_of(field)
    assert "300 distinct values" in str(e.value)
    with pytest.raises(api.Sw2dError):
        api.manning_classes_of(field[:65], max_classes=64)
    api.manning_classes_of(field[:64], max_classes=64)
    for bad in (np.nan, -0.01, np.inf):
        with pytest.raises(api.Sw2dError):
            api.manning_classes_of(np.array([0.03, bad]))


def test_manning_field_shape_is_checked(lib):
    m = _model()
    m.set_manning_field(np.full((6, 5), 0.03))
    m.set_manning_field(None)
    with pytest.raises(ValueError):
        m.set_manning_field(np.full((5, 6), 0.03))
    assert lib.calls == ["sw2d_set_manning_field"] * 2


def test_coupling_faces_of_edge_cases():
    # no lake: no faces; all lake: no faces (only non-lake cells test sides);
    # a lake cell in a corner: its neighbours on the edges see it only along
    # the sides the reference tests there
    assert all(len(a) == 0 for a in api.coupling_faces_of(np.zeros((5, 6), np.int32)))
    assert all(len(a) == 0 for a in api.coupling_faces_of(np.ones((5, 6), np.int32)))
    m = np.zeros((5, 6), np.int32)
    m[0, 0] = 1
    side, fi, fj, cell = api.coupling_faces_of(m)
    assert len(side) == 2 and sorted(cell.tolist()) == [1, 6]
    with pytest.raises(api.Sw2dError):
        api.coupling_faces_of(np.zeros((0, 4), np.int32))

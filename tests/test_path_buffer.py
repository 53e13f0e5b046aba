"""PathBuffer (crates/path/src/path_buffer.rs) as the batched container: paths appended by
builders come back unchanged, the batch layout is the C ABI's, and attribute tables line up
with the points."""

import numpy as np

from lyon_gb300.path import Path, PathBatch, PathBuilder, Verb
from lyon_gb300.path_buffer import PathBuffer


def test_builders_append_and_index():
    buf = PathBuffer()
    b = buf.builder()
    assert b.begin((0, 0)) == 0
    assert b.line_to((1, 0)) == 1
    b.quadratic_bezier_to((2, 0), (2, 1))
    b.end(True)
    i0 = b.build()
    b = buf.builder()
    b.add_circle((5.0, 5.0), 2.0)
    i1 = b.build()
    assert (i0, i1) == (0, 1) and len(buf) == 2 and not buf.is_empty()
    assert list(buf.get(0).verbs) == [Verb.BEGIN, Verb.LINE_TO, Verb.QUADRATIC_TO, Verb.CLOSE]
    assert buf.get(0).num_points == 5
    ref = PathBuilder()
    ref.add_circle((5.0, 5.0), 2.0)
    assert np.array_equal(buf.get(1).points, ref.build().points)
    batch = buf.as_batch()
    assert isinstance(batch, PathBatch) and batch.num_paths == 2
    assert np.array_equal(batch.path(1).points, buf.get(1).points)
    assert list(buf.indices()) == [0, 1]


def test_from_paths_and_clear():
    paths = [Path.from_arrays([Verb.BEGIN, Verb.LINE_TO, Verb.END], [[0, 0], [i, 1]])
             for i in range(5)]
    buf = PathBuffer.from_paths(paths)
    assert len(buf) == 5
    assert all(np.array_equal(a.points, b.points) for a, b in zip(buf, paths))
    buf.clear()
    assert buf.is_empty()


def test_attributes_table():
    buf = PathBuffer()
    b = buf.builder().with_attributes(2)
    b.begin((0, 0), [1, 2])
    b.line_to((1, 0), [3, 4])
    b.cubic_bezier_to((1, 1), (0, 1), (0, 2), [5, 6])
    b.end(True)
    b.build()
    pb = buf.builder()
    pb.begin((9, 9))
    pb.line_to((8, 8))
    pb.end(False)
    pb.build()
    t = buf.attribute_table()
    assert t.shape == (len(buf.as_batch().points), 2)
    # begin, line, cubic (two control rows and the end point), Close's repeated first point.
    want = np.array([[1, 2], [3, 4], [5, 6], [5, 6], [5, 6], [1, 2]], np.float32)
    assert np.array_equal(t[:6], want)
    assert np.array_equal(t[6:], np.zeros((2, 2), np.float32))
    assert buf.num_attributes(0) == 2 and buf.num_attributes(1) == 0

"""DataTracer (quantax/utils/data.py:8-147): the series the drivers trace."""
import io

import numpy as np

from quantax_gb300.utils import DataTracer


def test_data_tracer_series_and_statistics():
    d = DataTracer()
    assert d.uncertainty() is None
    for x in (1.0, 2.0, 4.0):
        d.append(x)
    np.testing.assert_array_equal(d.time, [0, 1, 2])  # default times count up from 0
    d.append(3.0, time=10.5)
    np.testing.assert_array_equal(np.asarray(d), [1.0, 2.0, 4.0, 3.0])
    assert d[2] == 4.0 and len(d) == 4 and d.time[-1] == 10.5
    assert d.mean() == 2.5
    x = d.data
    assert np.isclose(d.uncertainty(), np.sqrt(np.sum((x - 2.5) ** 2) / 4 / 3))
    t, v = d.batched(batch=3)  # the trailing partial group is dropped
    np.testing.assert_allclose(v, [7.0 / 3])
    np.testing.assert_allclose(t, [1.0])
    buf = io.BytesIO()
    d.save(buf)
    buf.seek(0)
    np.testing.assert_array_equal(np.load(buf), x)

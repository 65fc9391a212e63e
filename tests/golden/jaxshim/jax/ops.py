import numpy as _np


def segment_sum(data, segment_ids, num_segments=None, **k):
    data = _np.asarray(data)
    out = _np.zeros((num_segments,) + data.shape[1:], dtype=data.dtype)
    _np.add.at(out, _np.asarray(segment_ids), data)
    return out

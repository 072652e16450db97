"""
CPU restatement of the reference's frame ingest: DaxReader.loadAFrame
(sa_library/datareader.py:232-243), FrameReader.loadAFrame
(sa_library/analysis_io.py:243-260) and padArray (sa_library/fitting.py:
112-132).

TEST INFRASTRUCTURE ONLY: the checker for the GPU ingest in tests/.
Product code never imports this module.

Pinned by tests/golden/g_ingest.npz, made by
tests/golden/make_golden_ingest.py with the reference's own Python readers
on synthetic .dax movies.
"""
import numpy

from oracle.finder import pad_array


def dax_frame(raw_frames, index, bigendian):
    """Frame `index` of raw file-order uint16 frames, in native order."""
    frame = numpy.array(raw_frames[index], dtype=numpy.uint16)
    if bigendian:
        frame.byteswap(True)
    return frame


def load_frame(frame, offset, gain, rqe):
    """(frame - offset) * (gain * rqe), values below 1 set to 1."""
    out = (frame - offset) * (gain * rqe)
    mask = out < 1.0
    if numpy.sum(mask) > 0:
        out[mask] = 1.0
    return out


def ingest(raw_frames, bigendian, offset, gain, rqe, pad):
    return numpy.stack([pad_array(load_frame(dax_frame(raw_frames, i, bigendian), offset, gain, rqe), pad)
                        for i in range(len(raw_frames))])

"""
Frame readers that convert camera frames to photo-electrons on the GPU, as
the reference's FrameReader / FrameReaderStd / FrameReaderSCMOS
(sa_library/analysis_io.py:217-295) and loadCMOSCalibration (:35-77).

loadAFrame(n) returns the reference's frame: (frame - offset) * (gain *
rqe) with values below 1 set to 1, computed by the fused ingest kernel
(saIngestFrames) and copied back.  loadFramesPadded(first, count, pad)
does the same for a batch of frames and also mirror-pads them
(padArray, sa_library/fitting.py:112-132), leaving them on the GPU for the
batched peak finder (BatchPeakFinder.newImages takes the device address).
"""
import ctypes

import numpy

from . import datareader, loadclib


class AnalysisIOException(Exception):
    pass


def loadCMOSCalibration(filename, verbose=False):
    """[offset, variance, gain, rqe] from a numpy.save'd calibration (the
    v0, v1 and v2 layouts the reference reads)."""
    data = numpy.load(filename, allow_pickle=True)
    if len(data) == 3:
        rqe = numpy.ones_like(data[0])
        return list(map(numpy.transpose, list(data) + [rqe]))
    if len(data) == 4 and data[3] == 1:
        return list(data[:3]) + [numpy.ones_like(data[0])]
    if len(data) == 5 and data[4] == 2:
        return list(data[:4])
    raise AnalysisIOException("Unknown sCMOS data format.")


class FrameReader(object):

    def __init__(self, movie_file=None, parameters=None, **kwds):
        super(FrameReader, self).__init__(**kwds)
        self.gain = None
        self.offset = None
        self.parameters = parameters
        self.rqe = 1.0
        self.movie_data = datareader.inferReader(movie_file)
        self.clib = loadclib.load()
        self._ih = {}

    def close(self):
        self.movie_data.close()
        for h in self._ih.values():
            self.clib.saIngestCleanup(h)
        self._ih = {}

    def filmSize(self):
        return self.movie_data.filmSize()

    def _handle(self, pad):
        if pad not in self._ih:
            w, h, _ = self.movie_data.filmSize()
            scale = self.gain * self.rqe
            off_a = numpy.ascontiguousarray(numpy.broadcast_to(self.offset, (h, w)), dtype=numpy.float64) \
                if numpy.ndim(self.offset) else None
            sc_a = numpy.ascontiguousarray(numpy.broadcast_to(scale, (h, w)), dtype=numpy.float64) \
                if numpy.ndim(scale) else None
            ih = self.clib.saIngestCreate(
                h, w, int(pad), None if off_a is None else off_a.ctypes.data_as(ctypes.c_void_p),
                None if sc_a is None else sc_a.ctypes.data_as(ctypes.c_void_p),
                0.0 if off_a is not None else float(self.offset), 1.0 if sc_a is not None else float(scale), 1)
            if not ih:
                raise AnalysisIOException(loadclib.last_error())
            self._ih[pad] = ih
        return self._ih[pad]

    def _ingest(self, first, count, pad):
        raw = numpy.ascontiguousarray(self.movie_data.loadRaw(first, count))
        ih = self._handle(pad)
        if self.clib.saIngestFrames(ih, raw.ctypes.data_as(ctypes.c_void_p), count, 16,
                                    int(self.movie_data.bigendian), 0, None) != 0:
            raise AnalysisIOException(loadclib.last_error())
        return ih

    def loadAFrame(self, frame_number):
        ih = self._ingest(frame_number, 1, 0)
        w, h, _ = self.movie_data.filmSize()
        out = numpy.zeros((h, w))
        self.clib.saIngestGetFrames(ih, out)
        return out

    def loadFramesPadded(self, first, count, pad):
        """Device address of count converted, mirror-padded frames
        (count x (h + 2 pad) x (w + 2 pad) doubles), valid until the next
        call with the same pad."""
        return self.clib.saIngestResultDevice(self._ingest(first, count, pad))


class FrameReaderStd(FrameReader):
    """A camera with one gain (ADU / e-) and offset (ADU)."""

    def __init__(self, camera_gain=None, camera_offset=None, **kwds):
        super(FrameReaderStd, self).__init__(**kwds)
        if camera_gain is None:
            self.gain = 1.0 / self.parameters.getAttr("camera_gain")
            self.offset = self.parameters.getAttr("camera_offset")
        else:
            self.gain = 1.0 / camera_gain
            self.offset = camera_offset


class FrameReaderSCMOS(FrameReader):
    """A sCMOS camera: per-pixel offset, gain and relative QE."""

    def __init__(self, calibration_file=None, **kwds):
        super(FrameReaderSCMOS, self).__init__(**kwds)
        if calibration_file is None:
            calibration_file = self.parameters.getAttr("camera_calibration")
        [self.offset, variance, gain, rqe] = loadCMOSCalibration(calibration_file)
        self.gain = 1.0 / gain
        self.rqe = 1.0 / rqe

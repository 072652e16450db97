"""
GPU image-analysis utilities behind the reference's
sa_library/ia_utilities_c.py:

  MaximaFinder (:132-250): same constructor arguments, findMaxima(images,
      want_height) and resetTaken(); the taken counts live on the GPU
      (saMaxima* in include/sa_finder.h), getTaken() copies them back;
  markDimmerPeaks, markLowSignificancePeaks, runningIfHasNeighbors and
      KDTree.nearest (:252-465): the post-fit culling, same arguments and
      in-place status updates, neighbour queries on the GPU.

The reference-layout entry points saCalcMaxPeaks / saFindLocalMaxima
(flmData, host arrays) are reached through FlmData below.
"""
import ctypes

import numpy

from . import loadclib


RUNNING = 0
CONVERGED = 1
ERROR = 2


class FlmData(ctypes.Structure):
    """flmData, sa_library/ia_utilities.c:20-36."""
    _fields_ = [("margin", ctypes.c_int), ("n_peaks", ctypes.c_int), ("z_range", ctypes.c_int),
                ("xsize", ctypes.c_int), ("ysize", ctypes.c_int), ("zsize", ctypes.c_int),
                ("radius", ctypes.c_double), ("threshold", ctypes.c_double),
                ("z_values", ctypes.c_void_p), ("taken", ctypes.c_void_p), ("images", ctypes.c_void_p)]


class MaximaFinderException(Exception):
    pass


class MaximaFinder(object):

    def __init__(self, margin=None, n_duplicates=1, radius=None, threshold=None, z_range=None,
                 z_values=None, **kwds):
        super(MaximaFinder, self).__init__(**kwds)
        self.clib = loadclib.load()
        self.n_duplicates = n_duplicates
        self.n_planes = len(z_values)
        if z_range is None:
            z_range = self.n_planes
        # the +1 keeps maxima off the margin's edge (ia_utilities_c.py:162-171)
        self.c_zvalues = numpy.ascontiguousarray(numpy.array(z_values), dtype=numpy.float64)
        self.mh = self.clib.saMaximaCreate(int(margin + 1), int(z_range), float(radius), float(threshold),
                                           self.c_zvalues, self.n_planes, int(n_duplicates))
        if not self.mh:
            raise MaximaFinderException(loadclib.last_error())
        self.shape = None

    def findMaxima(self, images, want_height=False):
        assert (len(images) == self.n_planes), "Number of planes does not match number of Z planes."
        if self.shape is None:
            self.shape = images[0].shape
        for image in images:
            assert (image.shape[0] == self.shape[0]), "Unexpected image x size!"
            assert (image.shape[1] == self.shape[1]), "Unexpected image y size!"
            assert (image.flags['C_CONTIGUOUS']), "Image is not C contiguous!"
        stack = numpy.ascontiguousarray(numpy.stack(images), dtype=numpy.float64)
        counts = numpy.zeros(1, dtype=numpy.int32)
        n = self.clib.saMaximaFind(self.mh, stack.ctypes.data_as(ctypes.c_void_p), 0, self.shape[0],
                                   self.shape[1], 1, counts, 0.0)
        if n < 0:
            raise MaximaFinderException(loadclib.last_error())
        rows = numpy.zeros((max(n, 1), 4))
        self.clib.saMaximaGetPeaks(self.mh, rows)
        rows = rows[:n]
        x, y, z, h = (numpy.ascontiguousarray(rows[:, k]) for k in range(4))
        if want_height:
            return [x, y, z, h]
        return [x, y, z]

    def getTaken(self):
        if self.shape is None:
            return None
        out = numpy.zeros((self.n_planes,) + tuple(self.shape), dtype=numpy.int32)
        self.clib.saMaximaGetTaken(self.mh, out)
        return out

    def resetTaken(self):
        if self.shape is None:
            return
        if self.clib.saMaximaResetTaken(self.mh) != 0:
            raise MaximaFinderException(loadclib.last_error())

    def cleanup(self):
        if self.mh:
            self.clib.saMaximaCleanup(self.mh)
        self.mh = None


def calc_max_peaks(flm):
    """saCalcMaxPeaks on a filled FlmData."""
    return loadclib.load().saCalcMaxPeaks(ctypes.byref(flm))


def find_local_maxima(flm, z, y, x, h):
    """saFindLocalMaxima on a filled FlmData (reference argument order)."""
    loadclib.load().saFindLocalMaxima(ctypes.byref(flm), z, y, x, h)
    return flm.n_peaks


def _c(a, dtype):
    assert a.flags["C_CONTIGUOUS"], "array is not C contiguous!"
    assert a.dtype == dtype, "expected %s" % numpy.dtype(dtype)
    return a


def markDimmerPeaks(x, y, h, status, r_removal, r_neighbors):
    """Non-ERROR peaks with a brighter peak within r_removal become ERROR,
    CONVERGED peaks within r_neighbors of one become RUNNING (status is
    updated in place); returns the number removed."""
    lib = loadclib.load()
    n = lib.saMarkDimmerPeaks(_c(x, numpy.float64), _c(y, numpy.float64), _c(h, numpy.float64),
                              _c(status, numpy.int32), float(r_removal), float(r_neighbors), x.size)
    if n < 0:
        raise MaximaFinderException(loadclib.last_error())
    return n


def markLowSignificancePeaks(x, y, significance, status, minimum_significance, r_neighbors):
    lib = loadclib.load()
    n = lib.saMarkLowSignificancePeaks(_c(x, numpy.float64), _c(y, numpy.float64),
                                       _c(significance, numpy.float64), _c(status, numpy.int32),
                                       float(minimum_significance), float(r_neighbors), x.size)
    if n < 0:
        raise MaximaFinderException(loadclib.last_error())
    return n


def runningIfHasNeighbors(status, c_x, c_y, n_x, n_y, radius):
    lib = loadclib.load()
    lib.saRunningIfHasNeighbors(_c(c_x, numpy.float64), _c(c_y, numpy.float64), _c(n_x, numpy.float64),
                                _c(n_y, numpy.float64), _c(status, numpy.int32), float(radius), c_x.size, n_x.size)
    return status


class KDTree(object):
    """Nearest-point queries within a radius (the reference's C kd-tree
    wrapper); equal distances go to the lower index."""

    def __init__(self, x=None, y=None, **kwds):
        super(KDTree, self).__init__(**kwds)
        self.clib = loadclib.load()
        x = numpy.ascontiguousarray(x, dtype=numpy.float64)
        y = numpy.ascontiguousarray(y, dtype=numpy.float64)
        self.kd_tree = self.clib.saCreateKDTree(x, y, x.size)

    def cleanup(self):
        self.clib.saFreeKDTree(self.kd_tree)
        self.kd_tree = None

    def nearest(self, x, y, max_dist):
        x = numpy.ascontiguousarray(x, dtype=numpy.float64)
        y = numpy.ascontiguousarray(y, dtype=numpy.float64)
        dist = numpy.zeros(x.size, dtype=numpy.float64) - 1.0
        index = numpy.zeros(x.size, dtype=numpy.int32) - 1
        self.clib.saNearestKDTree(self.kd_tree, x, y, dist, index, float(max_dist), x.size)
        return [dist, index]

"""
Reader of the Zhuang lab .dax movie format (the reference's DaxReader,
sa_library/datareader.py:156-243, is the reader this replaces): the .inf
side file gives the frame size, frame count and byte order; frames are
uint16.

loadAFrame returns one frame in native byte order, as the reference does.
loadRaw returns consecutive frames exactly as stored (no byte swap), for
the GPU ingest, which swaps while it converts (saIngestFrames).
"""
import os
import re

import numpy


def read_inf(inf_filename):
    """The fields of a .inf side file as a dict of stripped strings: one
    "key = value" pair per line (lines without " = " are skipped)."""
    fields = {}
    with open(inf_filename, "r") as inf:
        for line in inf:
            key, sep, value = line.partition(" = ")
            if sep:
                fields[key.strip()] = value.strip()
    return fields


_DIMS = re.compile(r"^\s*(\d+)\s*x\s*(\d+)\s*$")


class DaxReader(object):
    """A .dax movie: frames of uint16 pixels, row-major, in the byte order
    the .inf file names ("... big endian" or "... little endian" in its
    data type; little endian when it names none).  The .inf's "frame
    dimensions = W x H" gives the width W (pixels per row) and height H, and
    "number of frames" the length."""

    def __init__(self, filename, verbose=False):
        self.filename = filename
        self.verbose = verbose
        self.inf_filename = os.path.splitext(filename)[0] + ".inf"
        fields = read_inf(self.inf_filename)
        dims = _DIMS.match(fields.get("frame dimensions", ""))
        if dims is None:
            raise IOError("%s: no 'frame dimensions = W x H' line" % self.inf_filename)
        self.image_width, self.image_height = int(dims.group(1)), int(dims.group(2))
        self.number_frames = int(fields.get("number of frames", "0"))
        order = " ".join(fields.values())
        self.bigendian = 1 if "big endian" in order else 0
        self.fileptr = open(filename, "rb") if os.path.exists(filename) else None

    def close(self):
        if self.fileptr:
            self.fileptr.close()
        self.fileptr = None

    def filmSize(self):
        return [self.image_width, self.image_height, self.number_frames]

    def loadRaw(self, first, count):
        """count frames from frame first, (count, height, width) uint16 as
        stored in the file."""
        assert 0 <= first and first + count <= self.number_frames, "frame range out of the movie"
        npix = self.image_height * self.image_width
        self.fileptr.seek(first * npix * 2)
        data = numpy.fromfile(self.fileptr, dtype=numpy.uint16, count=npix * count)
        return data.reshape(count, self.image_height, self.image_width)

    def loadAFrame(self, frame_number):
        frame = self.loadRaw(frame_number, 1)[0]
        if self.bigendian:
            frame.byteswap(True)
        return frame


def inferReader(filename, verbose=False):
    ext = os.path.splitext(filename)[1]
    if ext == ".dax":
        return DaxReader(filename, verbose=verbose)
    raise IOError("only .dax movies are read by this package (got %s)" % ext)

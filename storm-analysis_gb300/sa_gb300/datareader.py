"""
Reader of the Zhuang lab .dax movie format, as the reference's DaxReader
(sa_library/datareader.py:156-243): the .inf side file gives the frame
size, frame count and byte order; frames are uint16.

loadAFrame returns one frame in native byte order, as the reference does.
loadRaw returns consecutive frames exactly as stored (no byte swap), for
the GPU ingest, which swaps while it converts (saIngestFrames).
"""
import os
import re

import numpy


class DaxReader(object):

    def __init__(self, filename, verbose=False):
        self.filename = filename
        self.verbose = verbose
        dirname = os.path.dirname(filename)
        if len(dirname) > 0:
            dirname = dirname + "/"
        self.inf_filename = dirname + os.path.splitext(os.path.basename(filename))[0] + ".inf"
        self.image_height = None
        self.image_width = None
        self.number_frames = 0
        self.bigendian = 0
        size_re = re.compile(r'frame dimensions = ([\d]+) x ([\d]+)')
        length_re = re.compile(r'number of frames = ([\d]+)')
        endian_re = re.compile(r' (big|little) endian')
        with open(self.inf_filename, "r") as inf:
            for line in inf:
                m = size_re.match(line)
                if m:
                    self.image_height = int(m.group(2))
                    self.image_width = int(m.group(1))
                m = length_re.match(line)
                if m:
                    self.number_frames = int(m.group(1))
                m = endian_re.search(line)
                if m:
                    self.bigendian = 1 if m.group(1) == "big" else 0
        if not self.image_height:
            print("Could not determine image size, assuming 256x256.")
            self.image_height = 256
            self.image_width = 256
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

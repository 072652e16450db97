"""Frame ingest on the CPU: the oracle (oracle/ingest.py) and this
package's .dax reader against the golden fixture made with the reference's
own readers (tests/golden/make_golden_ingest.py)."""
import os

import numpy
import pytest

from oracle import ingest as I

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "g_ingest.npz")


@pytest.fixture(scope="module")
def g():
    return numpy.load(GOLDEN)


def write_dax(path, raw, bigendian):
    """raw: (n, h, w) uint16 frames as stored."""
    n, h, w = raw.shape
    raw.tofile(path)
    with open(os.path.splitext(path)[0] + ".inf", "w") as f:
        f.write("data type = 16 bit integers (binary, %s endian)\n" % ("big" if bigendian else "little"))
        f.write("frame dimensions = %d x %d\n" % (w, h))
        f.write("number of frames = %d\n" % n)


def test_oracle_matches_reference_readers(g):
    for tag, big in (("big", 1), ("little", 0)):
        assert numpy.array_equal(I.ingest(g["raw_" + tag], big, 100.0, 1.0 / 2.5, 1.0, 0), g["std_" + tag])
        assert numpy.array_equal(I.ingest(g["raw_" + tag], big, 100.0, 1.0 / 2.5, 1.0, 7), g["std_%s_pad7" % tag])
    sc = I.ingest(g["raw_big"], 1, g["offset"], 1.0 / g["gain"], 1.0 / g["rqe"], 11)
    assert numpy.array_equal(sc, g["scmos_big_pad11"])


def test_dax_reader_parses_and_swaps(g, tmp_path):
    from sa_gb300 import datareader
    for tag, big in (("big", 1), ("little", 0)):
        path = str(tmp_path / ("m_%s.dax" % tag))
        write_dax(path, g["raw_" + tag], big)
        rd = datareader.DaxReader(path)
        n, h, w = g["frames"].shape
        assert rd.filmSize() == [w, h, n] and rd.bigendian == big
        for i in range(n):
            assert numpy.array_equal(rd.loadAFrame(i), g["frames"][i])
        assert numpy.array_equal(rd.loadRaw(0, n), g["raw_" + tag])
        rd.close()

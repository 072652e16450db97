"""
The pupil-function PSF object of the reference's pupil-function analysis
(pupilfn/pupil_fn.py PupilFunction): the pupil function from a pickle file
('pf' complex128 size x size, 'pixel_size' and, for the geometry,
'wavelength', 'immersion_index', 'numerical_aperture' and 'geo_sim_pf'),
its C object (pupil_function_c.PupilFunction) for the fitter, and the
intensity PSF at a z (nanometers) for the peak finder.

zmin, zmax (nanometers) are the fit's z range as the caller gives them;
getZMin / getZMax return them unchanged.
"""
import pickle

import numpy

from . import pupil_function_c
from . import pupil_math


class PupilFunction(object):

    def __init__(self, pf_filename=None, zmin=None, zmax=None, pf_data=None, **kwds):
        super(PupilFunction, self).__init__(**kwds)
        self.zmax = zmax
        self.zmin = zmin
        if pf_data is None:
            with open(pf_filename, "rb") as fp:
                pf_data = pickle.load(fp)
        pf = pf_data["pf"]
        if pf.dtype != numpy.complex128:
            raise pupil_function_c.PupilFunctionException("The pupil function must be complex128.")
        self.pixel_size = pf_data["pixel_size"]
        self.pupil_size = pf.shape[0]
        cls = pupil_math.GeometrySim if pf_data.get("geo_sim_pf", False) else pupil_math.Geometry
        geo = cls(self.pupil_size, self.pixel_size, pf_data["wavelength"], pf_data["immersion_index"],
                  pf_data["numerical_aperture"])
        self.pupil_fn_c = pupil_function_c.PupilFunction(geo)
        self.pupil_fn_c.setPF(pf)

    def cleanup(self):
        self.pupil_fn_c.cleanup()

    def getCPointer(self):
        return self.pupil_fn_c.getCPointer()

    def getMargin(self):
        return int(self.getSize() / 2 + 2)

    def getPixelSize(self):
        return self.pixel_size

    def getPSF(self, z_value, shape=None, normalize=False):
        """The intensity PSF at z_value (nanometers), centred in an array of
        the given shape when one is given."""
        self.pupil_fn_c.translate(0.0, 0.0, 1.0e-3 * z_value)
        psf = pupil_math.intensity(self.pupil_fn_c.getPSF())
        if shape is not None:
            n = psf.shape[0]
            sx, sy = int(shape[0] / 2.0 - n / 2.0), int(shape[1] / 2.0 - n / 2.0)
            big = numpy.zeros((shape[0], shape[1]))
            big[sx:sx + n, sy:sy + n] = psf
            psf = big
        if normalize:
            psf = psf / numpy.sum(psf)
        return psf

    def getScaledZ(self, z):
        return z * 1.0e-3

    def getSize(self):
        return self.pupil_size

    def getZMax(self):
        return self.zmax

    def getZMin(self):
        return self.zmin

"""Emissivity models of the equatorial image (drop-in for kgeo.emissivities.Emissivity).

The constructor keeps the reference's keyword handling (kgeo/emissivities.py:38-72); the
profiles themselves are evaluated inside the image kernel (kgeo_gb300/csrc/kg_image.cuh).
Models on the GPU path: 'bpl', 'constant', 'glm', 'ring'. 'thermal' is accepted here and
refused by the image calls (it needs the B-field models, outside this package's scope).
"""

P1E_230 = -2.0
P2E_230 = -0.5
GAMMAOFF = -1.5
SIGMA_GLM = 0.5
R_RING = 4.5
SIGMA_RING = 0.3


class Emissivity(object):
    """Rest-frame emissivity as a function of r in the equatorial plane."""

    def __init__(self, emistype="bpl", **kwargs):
        self.emistype = emistype
        self.kwargs = kwargs
        self.emiscut_in = self.kwargs.get('emiscut_in', 0)
        self.emiscut_out = self.kwargs.get('emiscut_out', 1.e10)
        if self.emistype == 'thermal':
            self.Rb = float(self.kwargs.get('Rb', 5.0))
            self.ne0 = float(self.kwargs['ne0'])
            self.Te0 = float(self.kwargs['Te0'])
            self.B0 = float(self.kwargs['B0'])
            self.alpha_n = float(self.kwargs.get('alpha_n', 0.7))
            self.alpha_T = float(self.kwargs.get('alpha_T', 1.0))
            self.alpha_B = float(self.kwargs.get('alpha_B', 1.5))
            self.bfield_model = bool(self.kwargs.get('bfield_model', False))
        elif self.emistype == 'bpl':
            self.p1 = self.kwargs.get('p1', P1E_230)
            self.p2 = self.kwargs.get('p2', P2E_230)
        elif self.emistype == 'ring':
            self.mu_ring = self.kwargs.get('r_ring', R_RING)
            self.gamma_off = self.kwargs.get('gamma_off', 0)
            self.sigma = self.kwargs.get('sigma', SIGMA_RING)
        elif self.emistype == 'glm':
            self.mu_ring = False
            self.gamma_off = self.kwargs.get('gamma_off', GAMMAOFF)
            self.sigma = self.kwargs.get('sigma', SIGMA_GLM)
        elif self.emistype == 'constant':
            pass
        else:
            raise Exception("emistype %s not recognized in Emissivity!" % self.emistype)

"""Lab-frame velocity models of the equatorial image (drop-in for kgeo.velocities.Velocity).

The constructor keeps the reference's keyword handling (kgeo/velocities.py:23-67); the
four-velocities are evaluated inside the image kernel (kgeo_gb300/csrc/kg_image.cuh).
Models on the GPU path: 'zamo', 'infall', 'kep' / 'cunningham', 'subkep' /
'cunningham_subkep', 'general'. The others are accepted here and refused by the image calls.
"""

ELLISCO = 1.
VRISCO = 2
P1 = 6.
P2 = 2.
DD = 0.2
BETA = 0.3
CHI = -150 * 3.141592653589793 / 180.


class Velocity(object):
    """Lab-frame velocity as a function of r in the equatorial plane."""

    def __init__(self, veltype="kep", **kwargs):
        self.veltype = veltype
        self.kwargs = kwargs
        if self.veltype == 'zamo' or self.veltype == 'infall':
            pass
        elif self.veltype == 'kep' or self.veltype == 'cunningham':
            self.retrograde = self.kwargs.get('retrograde', False)
        elif self.veltype == 'subkep' or self.veltype == 'cunningham_subkep':
            self.retrograde = self.kwargs.get('retrograde', False)
            self.fac_subkep = self.kwargs.get('fac_subkep', 1)
        elif self.veltype == 'general':
            self.retrograde = self.kwargs.get('retrograde', False)
            self.fac_subkep = self.kwargs.get('fac_subkep', 1)
            self.beta_phi = self.kwargs.get('beta_phi', 1)
            self.beta_r = self.kwargs.get('beta_r', 1)
        elif self.veltype == 'gelles':
            self.gelles_beta = self.kwargs.get('gelles_beta', BETA)
            self.gelles_chi = self.kwargs.get('gelles_chi', CHI)
        elif self.veltype == 'simfit':
            self.ell_isco = self.kwargs.get('ell_isco', ELLISCO)
            self.vr_isco = self.kwargs.get('vr_isco', VRISCO)
            self.p1 = self.kwargs.get('p1', P1)
            self.p2 = self.kwargs.get('p2', P2)
            self.dd = self.kwargs.get('dd', DD)
        elif self.veltype in ('fromfile', 'driftframe'):
            pass
        else:
            raise Exception("veltype %s not recognized in Velocity!" % self.veltype)

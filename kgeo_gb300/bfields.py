"""Magnetic field models of the polarised equatorial image (drop-in for kgeo.bfields.Bfield).

The constructor keeps the reference's keyword handling and checks (kgeo/bfields.py:33-91);
the lab-frame field B^i is evaluated inside the image kernel (kgeo_gb300/csrc/kg_polar.cuh)
for every lab-frame model: 'rad', 'vert', 'tor', 'simple', 'simple_rm1', 'monopoleA',
'bz_guess', 'bz_monopole', 'bz_para', 'power', 'gen_power'. 'fromfile' (a tabulated field)
and the comoving-frame 'const_comoving' are accepted here and refused by the image calls.

'bz_monopole' evaluates the BZ radial function f(r) in closed form; the reference reads it
from a linearly interpolated table that it does not ship (kgeo/bfields.py:15-31).
"""
from . import _lib


class Bfield(object):
    """Magnetic field as a function of r in the equatorial plane."""

    def __init__(self, fieldtype="rad", **kwargs):
        self.fieldtype = fieldtype
        if self.fieldtype in ['rad', 'vert', 'tor', 'simple', 'simple_rm1', 'monopoleA', 'bz_monopole', 'bz_guess',
                              'bz_para', 'power', 'fromfile', 'gen_power']:
            self.fieldframe = 'lab'
        elif self.fieldtype in ['const_comoving']:
            self.fieldframe = 'comoving'
        else:
            raise Exception("fieldtype %s not recognized in Bfield!" % self.fieldtype)
        self.kwargs = kwargs
        if self.fieldtype in ['bz_monopole', 'bz_guess', 'bz_para']:
            self.secondorder_only = self.kwargs.get('secondorder_only', False)
            self.C = self.kwargs.get('C', 1)
        elif self.fieldtype in ['monopoleA']:
            self.omegafac = self.kwargs.get('omegafac', 0.5)
            self.C = self.kwargs.get('C', 1)
        elif self.fieldtype == 'power':
            self.secondorder_only = self.kwargs.get('secondorder_only', False)
            self.C = self.kwargs.get('C', 1)
            self.pval = self.kwargs.get('p', 1)
            self.usemono = self.kwargs.get('usemono', False)
        elif self.fieldtype == 'rad':
            self.Cr, self.Cvert, self.Cph = 1, 0, 0
        elif self.fieldtype == 'vert':
            self.Cr, self.Cvert, self.Cph = 0, 1, 0
        elif self.fieldtype == 'tor':
            self.Cr, self.Cvert, self.Cph = 0, 0, 1
        elif self.fieldtype == 'fromfile':
            self.filename = self.kwargs.get('file', None)
        elif self.fieldtype == 'gen_power':
            self.n_I = self.kwargs.get('n_I', 0)
            self.p_val = self.kwargs.get('p_val', 1)
            self.isAbove = self.kwargs.get('isAbove', True)
        else:
            self.Cr = self.kwargs.get('Cr', 0)
            self.Cvert = self.kwargs.get('Cvert', 0)
            self.Cph = self.kwargs.get('Cph', 0)
            if self.Cr == self.Cvert == self.Cph == 0.:
                raise Exception("all field coefficients are 0!")


def field_struct(bfield):
    """kgeo_bfield for a Bfield (this package's or the reference's object: only its
    attributes are read)."""
    ft = getattr(bfield, 'fieldtype', None)
    if getattr(bfield, 'fieldframe', 'lab') != 'lab':
        raise NotImplementedError("comoving-frame fields (%r) are not on the GPU image path" % (ft,))
    if ft not in _lib.BFIELD:
        raise NotImplementedError("B-field %r is not on the GPU image path" % (ft,))
    b = _lib.BField()
    b.field = _lib.BFIELD[ft]
    c = [0.0, 0.0, 0.0]
    if ft in ('rad', 'vert', 'tor', 'simple', 'simple_rm1'):
        c = [float(bfield.Cr), float(bfield.Cvert), float(bfield.Cph)]
    elif ft == 'monopoleA':
        c = [float(bfield.C), float(bfield.omegafac), 0.0]
    elif ft in ('bz_guess', 'bz_para'):
        c = [float(bfield.C), 0.0, 0.0]
    elif ft == 'bz_monopole':
        c = [float(bfield.C), 0.0, 0.0]
        b.flag = int(bool(bfield.secondorder_only))
    elif ft == 'power':
        c = [float(bfield.C), float(bfield.pval), 0.0]
        b.flag = int(bool(bfield.usemono))
    elif ft == 'gen_power':
        c = [float(bfield.n_I), float(bfield.p_val), 0.0]
        b.flag = int(bool(bfield.isAbove))
    for k in range(3):
        b.c[k] = c[k]
    return b

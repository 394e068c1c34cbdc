"""Model-update arithmetic of the inversion drivers through the host library
(sfwi_gb300/host/sfwi_host.h): the conjugate-gradient directions, the
stage-1 parabola step and the two model updates, with the state carried from
one iteration to the next in an object."""
import ctypes as C

import numpy as np

from . import su

_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)
_done = False


def _lib():
    global _done
    lib = su.host()
    if not _done:
        i, d = C.c_int, C.c_double
        lib.sfwi_stage1_direction.restype = d
        lib.sfwi_stage1_direction.argtypes = [i, i, i, _fp, _fp, _fp, _fp, _fp, _dp, _fp, _fp, _fp, _fp]
        lib.sfwi_stage1_alpha.restype = d
        lib.sfwi_stage1_alpha.argtypes = [d, d, d, C.c_float, C.c_float]
        lib.sfwi_stage1_update.restype = None
        lib.sfwi_stage1_update.argtypes = [i, i, d, _fp, _fp, _fp, _fp]
        lib.sfwi_stage2_direction.restype = d
        lib.sfwi_stage2_direction.argtypes = [i, i, i, _fp, _fp, _fp, _fp, _fp, _dp, _fp, _fp]
        lib.sfwi_stage2_update.restype = d
        lib.sfwi_stage2_update.argtypes = [i, i, d, d, _fp, _fp, _fp, _fp]
        _done = True
    return lib


def _p(a):
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_fp)


class CG:
    """Conjugate-gradient state of one inversion (the reference's pp_cg_old,
    ps_cg_old and beta_fenmu) on an allnx x allnz model."""

    def __init__(self, allnx, allnz):
        self.allnx, self.allnz = allnx, allnz
        self.old_pp = np.zeros((allnx, allnz), np.float32)
        self.old_ps = np.zeros((allnx, allnz), np.float32)
        self.beta_fenmu = C.c_double(0.0)

    def stage1(self, it, grad_pp, grad_ps, illum):
        """(beta, cg_pp, cg_ps, d_pp, d_ps): the preconditioned CG direction
        and its normalised copy for the line search."""
        g = [np.ascontiguousarray(a, np.float32) for a in (grad_pp, grad_ps, illum)]
        out = [np.empty((self.allnx, self.allnz), np.float32) for _ in range(4)]
        beta = _lib().sfwi_stage1_direction(self.allnx, self.allnz, it, *[_p(a) for a in g], _p(self.old_pp),
                                            _p(self.old_ps), C.byref(self.beta_fenmu), *[_p(a) for a in out])
        return (beta, *out)

    def stage2(self, it, grad_pp, grad_ps, illum):
        """(beta, grad_pp, grad_ps, cg_pp, cg_ps): the gradients with the
        layers above the cut zeroed, and the CG direction."""
        gp, gs = (np.array(a, np.float32, order="C") for a in (grad_pp, grad_ps))
        il = np.ascontiguousarray(illum, np.float32)
        cp, cs = (np.empty((self.allnx, self.allnz), np.float32) for _ in range(2))
        beta = _lib().sfwi_stage2_direction(self.allnx, self.allnz, it, _p(gp), _p(gs), _p(il), _p(self.old_pp),
                                            _p(self.old_ps), C.byref(self.beta_fenmu), _p(cp), _p(cs))
        return beta, gp, gs, cp, cs


def stage1_alpha(m0, m1, m2, step1=30.0, step2=150.0):
    return _lib().sfwi_stage1_alpha(m0, m1, m2, step1, step2)


def stage1_update(alpha, d_pp, d_ps, vp, vs):
    """vp, vs (float32, updated in place) -= alpha d; cut layers flattened"""
    d = [np.ascontiguousarray(a, np.float32) for a in (d_pp, d_ps)]
    _lib().sfwi_stage1_update(vp.shape[0], vp.shape[1], alpha, _p(d[0]), _p(d[1]), _p(vp), _p(vs))


def stage2_update(fenzi, fenmu, cg_pp, cg_ps, image_pp, image_ps):
    """image (float32, updated in place) -= (fenzi / fenmu) cg; returns alpha"""
    c = [np.ascontiguousarray(a, np.float32) for a in (cg_pp, cg_ps)]
    return _lib().sfwi_stage2_update(image_pp.shape[0], image_pp.shape[1], fenzi, fenmu, _p(c[0]), _p(c[1]),
                                     _p(image_pp), _p(image_ps))

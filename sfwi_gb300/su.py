"""SU record files and para_stage parameter files through the host library
(sfwi_gb300/host/sfwi_host.h): index a file into shots, read and write shot
gathers, read a parameter file."""
import ctypes as C
import os

import numpy as np

from . import _lib

HOST_LIB = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "libsfwi_host.so")
DRIVER = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "sfwi_fwi")


class Shot(C.Structure):
    _fields_ = [("no", C.c_int), ("ntr", C.c_int), ("sx", C.c_int), ("cx_min", C.c_int), ("cx_max", C.c_int),
                ("pos", C.c_longlong)]


class Para(C.Structure):
    _fields_ = [("dx", C.c_float), ("dz", C.c_float)] + \
               [(n, C.c_int) for n in ("pml", "allnx", "allnz", "minshot", "maxshot")] + \
               [(n, C.c_char * 1024) for n in ("vp", "vs", "rho", "rec_z", "rec_x", "outdir")] + \
               [("f0", C.c_float)] + [(n, C.c_int) for n in ("maxiter", "iter_round1", "sy", "gy", "light", "rbc",
                                                              "cpu_mem", "iointerval")]


_host = None


def host():
    global _host
    if _host is None:
        if not os.path.exists(HOST_LIB):
            raise OSError("%s is missing: run python -m sfwi_gb300.build" % HOST_LIB)
        lib = C.CDLL(HOST_LIB)
        lib.sfwi_su_index.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_float), C.POINTER(Shot), C.c_int,
                                      C.POINTER(C.c_int)]
        lib.sfwi_su_read.argtypes = [C.c_char_p, C.c_longlong, C.c_int, C.c_int, C.POINTER(C.c_float),
                                     C.POINTER(C.c_int)]
        lib.sfwi_su_write.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_int, C.POINTER(C.c_int),
                                      C.POINTER(C.c_float)]
        lib.sfwi_para_read.argtypes = [C.c_char_p, C.POINTER(Para)]
        _host = lib
    return _host


def index(path):
    """(nt, dt, [dict(no, ntr, sx, cx_min, cx_max, pos), ...])"""
    nt, dt, ns = C.c_int(), C.c_float(), C.c_int()
    if host().sfwi_su_index(path.encode(), C.byref(nt), C.byref(dt), None, 0, C.byref(ns)):
        raise OSError("cannot index %s" % path)
    arr = (Shot * max(ns.value, 1))()
    host().sfwi_su_index(path.encode(), C.byref(nt), C.byref(dt), arr, ns.value, C.byref(ns))
    shots = [{k: getattr(arr[i], k) for k, _ in Shot._fields_} for i in range(ns.value)]
    return nt.value, dt.value, shots


def read(path, pos, ntr, nt):
    """(records float32 [ntr, nt], gx int32 [ntr]) of ntr traces from trace `pos`."""
    dat = np.zeros((ntr, nt), np.float32)
    gc = np.zeros(ntr, np.int32)
    if host().sfwi_su_read(path.encode(), pos, ntr, nt, dat.ctypes.data_as(C.POINTER(C.c_float)),
                           gc.ctypes.data_as(C.POINTER(C.c_int))):
        raise OSError("cannot read %s" % path)
    return dat, gc


def write(path, sx, gc, dat, dt, append=False):
    dat = np.ascontiguousarray(dat, np.float32)
    gc = np.ascontiguousarray(gc, np.int32)
    ntr, nt = dat.shape
    if host().sfwi_su_write(path.encode(), int(append), ntr, nt, float(dt), int(sx),
                            gc.ctypes.data_as(C.POINTER(C.c_int)), dat.ctypes.data_as(C.POINTER(C.c_float))):
        raise OSError("cannot write %s" % path)


def read_para(path):
    p = Para()
    if host().sfwi_para_read(path.encode(), C.byref(p)):
        raise OSError("cannot read %s" % path)
    out = {}
    for k, _ in Para._fields_:
        v = getattr(p, k)
        out[k] = v.decode() if isinstance(v, bytes) else v
    return out


del _lib

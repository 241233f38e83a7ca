"""ctypes binding of the SunlightLB C API.

One :class:`Library` wraps any shared library that exports the SunlightLB API
of ``include/sunlightlb.h`` -- the GB300 library itself, and (in tests) the
CPU oracle or a build of the reference -- so the same driver code runs on all
of them.  It mirrors the SWIG Python module the reference builds
(src/SunlightLB.i, src/SunlightLB_setup.py): module-style functions taking the
system handle first (``lbstep(lb)``) and attribute access to every struct
field (``lb.tau = 0.8``, ``obj.frcx``), as in examples/sphere.py.
"""

import ctypes as C
import os

import numpy as np

LBReal = C.c_double


class LBObjStruct(C.Structure):
    pass


LBObjStruct._fields_ = [
    ("id", C.c_int),
    ("posx", LBReal), ("posy", LBReal), ("posz", LBReal),
    ("velx", LBReal), ("vely", LBReal), ("velz", LBReal),
    ("angx", LBReal), ("angy", LBReal), ("angz", LBReal),
    ("frcx", LBReal), ("frcy", LBReal), ("frcz", LBReal),
    ("trqx", LBReal), ("trqy", LBReal), ("trqz", LBReal),
    ("next_obj", C.POINTER(LBObjStruct)),
    ("base_obj", C.POINTER(LBObjStruct)),
]

# Fields of LBSys_struct in the reference order (reference src/sunlightlb.h:68-100)
_LBSYS_BASE = [
    ("w", C.POINTER(C.c_int)), ("c", C.POINTER(C.c_int)),
    ("a", C.POINTER(LBReal)),
    ("ux", C.POINTER(LBReal)), ("uy", C.POINTER(LBReal)), ("uz", C.POINTER(LBReal)),
    ("fx", C.POINTER(LBReal)), ("fy", C.POINTER(LBReal)), ("fz", C.POINTER(LBReal)),
    ("bx", C.POINTER(LBReal)), ("by", C.POINTER(LBReal)), ("bz", C.POINTER(LBReal)),
    ("esi", C.c_int), ("esj", C.c_int), ("esk", C.c_int), ("nnodes", C.c_int),
    ("step", C.c_int), ("status", C.c_int), ("changed_objects", C.c_int),
    ("objects_moving", C.c_int), ("skip_solid", C.c_int), ("stokes_flow", C.c_int),
    ("vel_corrected", C.c_int), ("monitoring", C.c_int),
    ("tau", LBReal), ("rho0", LBReal),
    ("vmeanx", LBReal), ("vmeany", LBReal), ("vmeanz", LBReal),
    ("psi", C.POINTER(LBReal)),
    ("rho", C.POINTER(LBReal)),
    ("name", C.c_char_p),
    ("rescale", LBReal),
    ("load_average", C.c_int),
    ("obj", C.POINTER(C.POINTER(LBObjStruct))),
    ("obj_head", C.POINTER(LBObjStruct)),
    ("mask", C.POINTER(C.c_int)),
    ("next_id", C.c_int),
]
_LBSYS_APPENDED = [("precision", C.c_int), ("priv", C.c_void_p)]


class LBSysBase(C.Structure):
    _fields_ = _LBSYS_BASE


class LBSysExt(C.Structure):
    _fields_ = _LBSYS_BASE + _LBSYS_APPENDED


_MPSYS_BASE = [
    ("lb", C.c_void_p),
    ("p", C.POINTER(LBReal)), ("newp", C.POINTER(LBReal)),
    ("step", C.c_int), ("objects_moving", C.c_int), ("to_be_initialised", C.c_int),
    ("alpha", LBReal), ("isoslice", LBReal), ("poffset", LBReal),
    ("p2bytemin", LBReal), ("p2bytemax", LBReal),
    ("name", C.c_char_p),
]
_MPSYS_APPENDED = [("adprob", LBReal), ("precision", C.c_int), ("priv", C.c_void_p)]


class MPSysBase(C.Structure):
    _fields_ = _MPSYS_BASE


class MPSysExt(C.Structure):
    _fields_ = _MPSYS_BASE + _MPSYS_APPENDED


# Status codes and verbosity flags (reference src/sunlightlb.h:39-49)
TRACE_ROUTINE_EXITS = 0x02
OBJECT_DETAILS = 0x04
MP_OBJECT_DETAILS = 0x04
FORCE_DETAILS = 0x08
POST_BBL = 42
POST_PROPAGATE = 47
POST_COLLIDE = 49
SLB_FP64, SLB_FP32, SLB_BF16 = 0, 1, 2

# Prototype table: name -> (restype code, [arg codes]).
#   L = LBSys, M = MPSys, O = LBObj, i = int, l = long, d = LBReal/double,
#   s = char*, p = void*, D = double* (numpy float64 array or None), v = void
PROTOS = {
    "newlb": ("L", "iiis"), "set_verbosity": ("v", "i"), "unset_verbosity": ("v", "i"),
    "about": ("v", ""), "wrpars": ("v", "L"), "wrlinks": ("v", "L"), "wrstats": ("v", "L"),
    "startclock": ("v", ""), "wrmon": ("v", "Ls"),
    "lbstep": ("v", "L"), "bbl": ("v", "L"), "bblforce": ("v", "L"),
    "propagate": ("v", "L"), "collide": ("v", "L"),
    "lookupobj": ("O", "Li"), "addobj": ("O", "L"), "zeroobj": ("v", "O"),
    "insertsubs": ("O", "Lsiiiiii"), "insertlist": ("O", "Ls"), "insertmask": ("O", "Lp"),
    "insertslab": ("O", "Ldddddd"), "insertsph": ("O", "Ldddd"),
    "insertcyl": ("O", "Lsddd"), "insertwall": ("O", "Lsi"),
    "flattenobj": ("O", "L"), "invertobj": ("O", "L"), "removeobjs": ("v", "L"),
    "wrobjs": ("v", "L"), "wrmap": ("v", "Ls"), "makemask": ("v", "L"),
    "vspread": ("v", "L"), "zerobf": ("v", "L"), "addbf": ("v", "Lddd"),
    "vset": ("v", "Liiiddd"), "countmask": ("i", "Ls"), "countfluid": ("i", "L"),
    "syncobjs": ("v", "L"),
    "lbsave": ("v", "Ls"), "lbload": ("v", "Ls"), "lbsavevel": ("v", "Lss"),
    "lbloadvel": ("v", "Lss"), "lbsavestr": ("v", "Lss"), "lbsaveobj": ("v", "Ls"),
    "lbloadobj": ("v", "Ls"), "lbsavefrc": ("v", "Lss"), "lbsavemap": ("v", "Lss"),
    "accvmean": ("v", "Ld"), "vzero": ("v", "L"), "vgrab": ("v", "Ld"), "vsave": ("v", "Ls"),
    "measure": ("v", "L"), "zeroforce": ("v", "L"), "normforce": ("v", "Ld"),
    "distribf": ("v", "L"), "wrmeas": ("v", "L"), "discrf": ("d", "L"),
    "mpstep": ("v", "M"), "newmp": ("M", "Ls"), "mpinit": ("v", "M"), "mpwrpars": ("v", "M"),
    "mprhoinit": ("v", "M"), "mpcheck": ("v", "M"), "mpmean": ("d", "M"),
    "mpmax": ("d", "M"), "mpmin": ("d", "M"), "mprescale": ("v", "Md"),
    "mpcopy": ("v", "MM"), "mpspread": ("d", "Ms"),
    "mpall": ("v", "Md"), "mpslab": ("v", "Mddddddd"), "mpwall": ("v", "Msid"),
    "mpsph": ("v", "Mddddd"), "mpcyl": ("v", "Msdddd"), "mplist": ("v", "Msd"),
    "mpsubs": ("v", "Msiiiiiid"),
    "mpvacfinit": ("v", "MMsi"), "mpvacfinit2": ("v", "MM"), "mpvacf": ("v", "MM"), "mpvacfwr": ("d", "MMsi"),
    "adall": ("v", "M"), "adnone": ("v", "M"), "adslab": ("v", "Mdddddd"),
    "adsph": ("v", "Mdddd"), "adcyl": ("v", "Msddd"), "adtotal": ("d", "Msi"),
    "adzero": ("v", "M"),
    # appended API
    "lbpull": ("v", "L"), "lbpush": ("v", "L"), "lbsteps": ("v", "Li"),
    "lbconverge": ("i", "Lidi"), "freelb": ("v", "L"), "lbgetstream": ("p", "L"),
    "lbsetstream": ("v", "Lp"), "lbkernelcount": ("l", ""), "lbtuning": ("i", "Lp"), "lbsettuning": ("i", "Lp"), "lblayout": ("i", "L"), "freemp": ("v", "M"),
    "lbsetvel": ("v", "LDDDD"), "lbsetveldev": ("v", "Lp"), "lbvelocity": ("v", "Lp"),
    "lbstate": ("v", "Lpp"), "lbsetstatedev": ("v", "Lpp"), "lbtranslate": ("v", "LOdddd"), "insertspheres": ("i", "LiDDDD"), "mptotal": ("d", "Ms"), "mpplane": ("d", "Msi"),
    "newbatch": ("p", ""), "batchadd": ("v", "pL"), "batchsteps": ("v", "pi"), "batchsize": ("i", "p"), "batchmode": ("v", "pi"),
    "freebatch": ("v", "p"), "mppull": ("v", "M"), "mppush": ("v", "M"),
}


class _Proxy:
    """Attribute access to the fields of a C struct behind a pointer."""

    _struct = None

    def __init__(self, lib, ptr):
        object.__setattr__(self, "_lib", lib)
        object.__setattr__(self, "_ptr", ptr)

    @property
    def _as_parameter_(self):
        return C.cast(self._ptr, C.c_void_p)

    def _s(self):
        return C.cast(self._ptr, C.POINTER(self._struct)).contents

    def __getattr__(self, name):
        s = self._s()
        if name in {f[0] for f in self._struct._fields_}:
            return getattr(s, name)
        raise AttributeError(name)

    def __setattr__(self, name, value):
        s = self._s()
        if name in {f[0] for f in self._struct._fields_}:
            setattr(s, name, value)
        else:
            object.__setattr__(self, name, value)

    def __eq__(self, other):
        return isinstance(other, _Proxy) and self.address == other.address

    def __hash__(self):
        return hash(self.address)

    @property
    def address(self):
        return C.cast(self._ptr, C.c_void_p).value


class LBObj(_Proxy):
    _struct = LBObjStruct


class LBSys(_Proxy):
    """Proxy of an LBSys; array fields are exposed as numpy views."""

    @property
    def _struct(self):
        return LBSysExt if self._lib.extended else LBSysBase

    def _s(self):
        return C.cast(self._ptr, C.POINTER(self._struct)).contents

    def _view(self, field, n, ctype=np.float64):
        ptr = getattr(self._s(), field)
        if not ptr:
            return None
        return np.ctypeslib.as_array(ptr, shape=(n,))

    def array(self, field):
        """numpy view of a per-node array field (a is 15*nnodes long)."""
        n = self.nnodes
        if field == "a":
            return self._view("a", 15 * n).reshape(n, 15)
        if field == "mask":
            return self._view("mask", n)
        if field == "obj":
            raw = getattr(self._s(), "obj")
            vp = C.cast(raw, C.POINTER(C.c_void_p))
            return np.ctypeslib.as_array(C.cast(vp, C.POINTER(C.c_uint64)), shape=(n,))
        return self._view(field, n)

    def pops(self):
        """Copy of the populations, shape (nnodes, 15), reference order."""
        if self._lib.has("lbpull"):  # a build of the reference keeps a on the host
            self._lib.call("lbpull", self)
        return self.array("a").copy()

    def objects(self):
        """Objects in list order (head first), as LBObj proxies."""
        out = []
        p = self._s().obj_head
        while p:
            out.append(LBObj(self._lib, p))
            p = p.contents.next_obj
        return out


class MPSys(_Proxy):
    @property
    def _struct(self):
        return MPSysExt if self._lib.extended else MPSysBase

    def _s(self):
        return C.cast(self._ptr, C.POINTER(self._struct)).contents

    def field(self):
        n = LBSys(self._lib, self._s().lb).nnodes
        return np.ctypeslib.as_array(self._s().p, shape=(n,))


_ARG = {"i": C.c_int, "l": C.c_long, "d": LBReal, "s": C.c_char_p, "p": C.c_void_p,
        "L": C.c_void_p, "M": C.c_void_p, "O": C.c_void_p, "D": C.c_void_p}
_RES = {"v": None, "i": C.c_int, "l": C.c_long, "d": LBReal, "p": C.c_void_p,
        "L": C.c_void_p, "M": C.c_void_p, "O": C.c_void_p}


class Library:
    """A loaded SunlightLB-API shared library.

    ``extended`` says whether its structs carry the appended fields of
    include/sunlightlb.h (the GB300 library and the oracle do; a build of the
    reference does not)."""

    def __init__(self, path, extended=True, mode=os.RTLD_LOCAL):
        self.path = path
        self.extended = extended
        self.dll = C.CDLL(path, mode=mode)
        self.funcs = {}
        for name, (res, args) in PROTOS.items():
            try:
                f = getattr(self.dll, name)
            except AttributeError:
                continue
            f.restype = _RES[res]
            f.argtypes = [_ARG[a] for a in args]
            self.funcs[name] = (f, res, args)

    def has(self, name):
        return name in self.funcs

    def call(self, name, *args):
        if name not in self.funcs:
            raise AttributeError(f"{os.path.basename(self.path)} does not export {name}")
        f, res, codes = self.funcs[name]
        conv = []
        keep = []
        for code, a in zip(codes, args):
            if code == "s":
                conv.append(a.encode() if isinstance(a, str) else a)
            elif code == "D":
                if a is None:
                    conv.append(None)
                else:
                    arr = np.ascontiguousarray(a, dtype=np.float64)
                    keep.append(arr)
                    conv.append(arr.ctypes.data)
            elif code in "LMO":
                conv.append(None if a is None else a._as_parameter_)
            else:
                conv.append(a)
        r = f(*conv)
        if res == "L":
            return LBSys(self, r) if r else None
        if res == "M":
            return MPSys(self, r) if r else None
        if res == "O":
            return LBObj(self, r) if r else None
        return r

    def __getattr__(self, name):
        if name.startswith("_") or name not in PROTOS:
            raise AttributeError(name)
        return lambda *a: self.call(name, *a)

    def globals(self):
        """Name -> callable for every exported API function (SWIG style)."""
        return {n: (lambda n: (lambda *a: self.call(n, *a)))(n) for n in self.funcs}

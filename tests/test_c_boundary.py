"""The C boundary, compiled: struct layouts against the reference header,
and a C driver linked against the library.

1. offsetof / sizeof of every field of LBObj_struct, LBSys_struct and
   MPSys_struct, printed by a C program compiled once against the
   reference's header (src/sunlightlb.h:53-121) and once against
   include/sunlightlb.h: the reference's fields must sit at the same
   offsets with the same sizes, and the appended fields after them.  The
   ctypes binding must agree with the compiler on include/sunlightlb.h.
2. tests/drivers/sphere_drag.c, a plain C driver of the reference API,
   compiled with gcc against include/sunlightlb.h and linked with
   -lsunlightlb (the library's soname, libsunlightlb.so.1) and, separately,
   against the CPU oracle.  It links here; on a GPU its output and files
   equal the oracle build's byte for byte (FP64 populations).

The reference checkout is $SLB_REFERENCE (default /root/reference); tests
that need its header skip when it is absent.
"""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")
DRIVER = os.path.join(ROOT, "tests", "drivers", "sphere_drag.c")
REF_SRC = os.path.join(os.environ.get("SLB_REFERENCE", "/root/reference"), "src")

FIELDS = {
    "LBObj_struct": ["id", "posx", "posy", "posz", "velx", "vely", "velz", "angx", "angy", "angz",
                     "frcx", "frcy", "frcz", "trqx", "trqy", "trqz", "next_obj", "base_obj"],
    "LBSys_struct": ["w", "c", "a", "ux", "uy", "uz", "fx", "fy", "fz", "bx", "by", "bz", "esi", "esj",
                     "esk", "nnodes", "step", "status", "changed_objects", "objects_moving",
                     "skip_solid", "stokes_flow", "vel_corrected", "monitoring", "tau", "rho0",
                     "vmeanx", "vmeany", "vmeanz", "psi", "rho", "name", "rescale", "load_average",
                     "obj", "obj_head", "mask", "next_id"],
    "MPSys_struct": ["lb", "p", "newp", "step", "objects_moving", "to_be_initialised", "alpha",
                     "isoslice", "poffset", "p2bytemin", "p2bytemax", "name"],
}
APPENDED = {"LBObj_struct": [], "LBSys_struct": ["precision", "priv"],
            "MPSys_struct": ["adprob", "precision", "priv"]}


def _gcc():
    cc = shutil.which(os.environ.get("CC", "gcc"))
    if cc is None:
        pytest.skip("no C compiler")
    return cc


def layout(include_dir, appended, tmp_path, tag):
    """{struct: {field: (offset, size)}} from a program compiled against
    the sunlightlb.h in include_dir."""
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "sunlightlb.h"', "int main(void) {"]
    for st, names in FIELDS.items():
        for f in names + (APPENDED[st] if appended else []):
            lines.append(f'  printf("{st} {f} %zu %zu\\n", offsetof(struct {st}, {f}), '
                         f'sizeof(((struct {st} *)0)->{f}));')
        lines.append(f'  printf("{st} sizeof %zu 0\\n", sizeof(struct {st}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / f"layout_{tag}.c"
    exe = tmp_path / f"layout_{tag}"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run([_gcc(), "-std=gnu99", "-I", include_dir, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    res = {}
    for line in out.splitlines():
        st, f, off, size = line.split()
        res.setdefault(st, {})[f] = (int(off), int(size))
    return res


def test_struct_layout_equals_reference_header(tmp_path):
    if not os.path.exists(os.path.join(REF_SRC, "sunlightlb.h")):
        pytest.skip("reference header not available (set SLB_REFERENCE)")
    ref = layout(REF_SRC, False, tmp_path, "ref")
    mine = layout(INC, True, tmp_path, "mine")
    for st, names in FIELDS.items():
        for f in names:
            assert mine[st][f] == ref[st][f], (st, f, mine[st][f], ref[st][f])
        last_ref = max(o + s for o, s in (ref[st][f] for f in names))
        for f in APPENDED[st]:
            assert mine[st][f][0] >= last_ref, (st, f)
        if not APPENDED[st]:
            assert mine[st]["sizeof"] == ref[st]["sizeof"]


def test_ctypes_binding_equals_compiled_layout(tmp_path):
    from sunlightlb_gb300.binding import LBObjStruct, LBSysExt, MPSysExt
    mine = layout(INC, True, tmp_path, "mine")
    for st, cls in (("LBObj_struct", LBObjStruct), ("LBSys_struct", LBSysExt), ("MPSys_struct", MPSysExt)):
        for f, _ in cls._fields_:
            assert getattr(cls, f).offset == mine[st][f][0], (st, f)
        assert C_sizeof(cls) == mine[st]["sizeof"][0]


def C_sizeof(cls):
    import ctypes
    return ctypes.sizeof(cls)


def build_driver(tmp_path, which):
    """Compile the C driver against include/sunlightlb.h and link it with
    the GPU library (-lsunlightlb, resolved through its soname) or the
    oracle."""
    from sunlightlb_gb300 import build as b
    exe = tmp_path / f"sphere_drag_{which}"
    if which == "gpu":
        if not os.path.exists(b.LIB):
            b.build()
        libdir = tmp_path / "lib"
        libdir.mkdir(exist_ok=True)
        for name in ("libsunlightlb.so", "libsunlightlb.so.1"):
            link = libdir / name
            if not link.exists():
                link.symlink_to(b.LIB)
        cmd = [_gcc(), "-std=gnu99", "-O2", "-I", INC, DRIVER, "-o", str(exe), "-L", str(libdir),
               "-lsunlightlb", "-Wl,-rpath," + str(libdir), "-lm"]
    else:
        orc = os.path.join(ROOT, "oracle", "liboracle.so")
        if not os.path.exists(orc):
            b.build_oracle(with_reference=False)
        cmd = [_gcc(), "-std=gnu99", "-O2", "-I", INC, DRIVER, "-o", str(exe), orc,
               "-Wl,-rpath," + os.path.dirname(orc), "-lm"]
    subprocess.run(cmd, check=True)
    return exe


def test_c_driver_links_against_library(tmp_path):
    """The driver compiles against the header and links with -lsunlightlb;
    the executable records the reference's soname."""
    exe = build_driver(tmp_path, "gpu")
    out = subprocess.run(["readelf", "-d", str(exe)], capture_output=True, text=True)
    if out.returncode == 0:
        assert "libsunlightlb.so.1" in out.stdout
    build_driver(tmp_path, "oracle")


def run_driver(exe, outdir, steps):
    outdir.mkdir()
    r = subprocess.run([str(exe), str(outdir), str(steps)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    values = [l for l in r.stdout.splitlines()
              if l.split()[:1] and l.split()[0] in ("step", "vmean", "force", "torque", "discrf")]
    files = {p.name: p.read_bytes() for p in sorted(outdir.iterdir())}
    return values, files


@pytest.mark.gpu
def test_c_driver_on_gpu_equals_oracle(tmp_path):
    gpu_exe = build_driver(tmp_path, "gpu")
    orc_exe = build_driver(tmp_path, "oracle")
    vg, fg = run_driver(gpu_exe, tmp_path / "g", 300)
    vo, fo = run_driver(orc_exe, tmp_path / "o", 300)
    assert len(vg) == 5
    assert vg[0] == vo[0]
    # mean flow and forces are reductions (summation order differs on the
    # GPU): 1e-12 relative; the files are byte-identical
    for lg, lo in zip(vg[1:], vo[1:]):
        a = [float(v) for v in lg.split()[1:]]
        b = [float(v) for v in lo.split()[1:]]
        scale = max(abs(v) for v in b) or 1.0
        assert max(abs(x - y) for x, y in zip(a, b)) <= 1e-12 * scale, (lg, lo)
    assert fg.keys() == fo.keys() == {"drag.map", "drag.frc", "drag.vel", "drag.obj"}
    for k in fg:
        assert fg[k] == fo[k], k

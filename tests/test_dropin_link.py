"""The drop-in boundary at the real caller: the reference's own Cython extension (pawpyc.pyx,
unmodified) compiled and linked against libpawpy_gpu.so as a maintainer would link it
(oracle/Makefile, target dropin), with every reference-named entry point the library defines
renamed inside the reference objects. Checks, without a GPU, that the extension needs the
library and that each of those entry points, looked up from the extension, is the library's
code. Skipped where the reference sources, Cython or binutils are absent.
"""

import ctypes
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

REFERENCE = os.environ.get("PAWPY_REFERENCE", "/root/reference")
REFDIR = os.path.join(REFERENCE, "pawpyseed", "core")
LIB = os.path.join(ROOT, "pawpyseed_gb300", "lib", "libpawpy_gpu.so")
EXT = os.path.join(ROOT, "oracle", "_ref", "dropin", "pawpyc.so")


class _DlInfo(ctypes.Structure):
    _fields_ = [("dli_fname", ctypes.c_char_p), ("dli_fbase", ctypes.c_void_p),
                ("dli_sname", ctypes.c_char_p), ("dli_saddr", ctypes.c_void_p)]


def _library_entry_points():
    out = subprocess.run(["nm", "-D", "--defined-only", LIB], capture_output=True, text=True, check=True).stdout
    names = [ln.split()[-1] for ln in out.splitlines() if ln.strip()]
    return sorted(n for n in names if not n.startswith("pawpy_gpu_") and not n.startswith("_"))


@pytest.mark.skipif(not os.path.exists(os.path.join(REFDIR, "pawpyc.pyx")), reason="reference sources absent")
@pytest.mark.skipif(shutil.which("cython") is None or shutil.which("objcopy") is None,
                    reason="cython or binutils absent")
def test_reference_extension_links_against_the_library():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "dropin", "REFDIR=" + REFDIR], check=True,
                   capture_output=True)
    needed = subprocess.run(["readelf", "-d", EXT], capture_output=True, text=True, check=True).stdout
    assert "[libpawpy_gpu.so]" in needed
    names = _library_entry_points()
    # the band-projection entry points and those of the aug_recip and real-space methods
    for n in ("pseudoprojection", "get_projector_list", "setup_projections", "onto_projector", "overlap_setup_real",
              "compensation_terms", "fft3d", "overlap_setup_recip", "compensation_terms_recip", "realspace_state",
              "ae_chg_density", "project_realspace_state"):
        assert n in names
    undefined = subprocess.run(["nm", "-D", "--undefined-only", EXT], capture_output=True, text=True,
                               check=True).stdout.split()
    defined = subprocess.run(["nm", "--defined-only", EXT], capture_output=True, text=True, check=True).stdout
    ext = ctypes.CDLL(EXT)
    dl = ctypes.CDLL(None)
    lib_real = os.path.realpath(LIB)
    for n in names:
        # not defined by the extension (the reference's own definition was renamed) ...
        assert n in undefined or (" T " + n + "\n") not in defined, n
        # ... and resolved, from the extension's scope, to the library's code
        info = _DlInfo()
        assert dl.dladdr(ctypes.cast(getattr(ext, n), ctypes.c_void_p), ctypes.byref(info)) != 0
        assert os.path.realpath(info.dli_fname.decode()) == lib_real, (n, info.dli_fname)
    # the reference's definitions of the path entry points are still in the extension, renamed
    assert "pawpy_ref_pseudoprojection" in defined and "pawpy_ref_setup_projections" in defined

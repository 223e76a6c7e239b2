"""ctypes wrapper of the serial C interface, with the same module-level API as
the reference's serial_interface/api/chimescalc_serial_py.py:

    import chimes_calculator_gb300.chimescalc_serial_py as wrapper_py
    wrapper_py.chimes_wrapper = wrapper_py.init_chimes_wrapper(path_to_libchimescalc)
    wrapper_py.set_chimes()
    wrapper_py.init_chimes(param_file, rank)
    fx, fy, fz, stress, energy = wrapper_py.calculate_chimes(natoms, x, y, z, types, ca, cb, cc,
                                                             energy, fx, fy, fz, stress)

init_chimes_wrapper() with no argument loads the in-tree libchimescalc.so.
calculate_chimes adds into the energy and forces it is given and returns the
updated ctypes arrays and energy, as the reference wrapper does (:43-99).
"""

import ctypes

from . import _lib

chimes_wrapper = None


def init_chimes_wrapper(lib_name=None):
    """Loads the library (the reference's init_chimes_wrapper, :24-25)."""
    if lib_name is None or lib_name == _lib.LIB_PATH:
        return _lib.load()
    lib = ctypes.CDLL(lib_name)
    for name, (res, args) in _lib.SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is not None:
            fn.restype, fn.argtypes = res, args
    return lib


def set_chimes(small=False):
    """Selects the static calculator instance (:27-30); small allows replication."""
    chimes_wrapper.set_chimes_serial(int(bool(small)))


def init_chimes(param_file, rank=0):
    """Reads the parameter file into the static instance (:33-40)."""
    in_rank = ctypes.c_int(rank)
    chimes_wrapper.init_chimes_serial(param_file.encode(), ctypes.byref(in_rank))


def calculate_chimes(natoms, xcrd, ycrd, zcrd, atmtyps, cell_a, cell_b, cell_c, energy, fx, fy, fz, stress):
    """Energy, forces and stress of one configuration (:43-99).  Returns the
    updated (fx, fy, fz, stress) ctypes arrays and the energy."""
    encoded = [atmtyps[i].encode() for i in range(natoms)]
    in_xcrd = (ctypes.c_double * natoms)(*xcrd)
    in_ycrd = (ctypes.c_double * natoms)(*ycrd)
    in_zcrd = (ctypes.c_double * natoms)(*zcrd)
    in_atmtyps = (ctypes.c_char_p * natoms)(*encoded)
    in_cell_a = (ctypes.c_double * 3)(*cell_a)
    in_cell_b = (ctypes.c_double * 3)(*cell_b)
    in_cell_c = (ctypes.c_double * 3)(*cell_c)
    in_energy = ctypes.c_double(energy)
    in_fx = (ctypes.c_double * natoms)(*fx)
    in_fy = (ctypes.c_double * natoms)(*fy)
    in_fz = (ctypes.c_double * natoms)(*fz)
    in_stress = (ctypes.c_double * 9)(*stress)
    chimes_wrapper.calculate_chimes(natoms, in_xcrd, in_ycrd, in_zcrd, in_atmtyps, in_cell_a, in_cell_b, in_cell_c,
                                    ctypes.byref(in_energy), in_fx, in_fy, in_fz, in_stress)
    return in_fx, in_fy, in_fz, in_stress, in_energy.value

"""ctypes mirror of ``tomo_spec`` (include/tomography.h) and spec helpers.

The reference fixes its problem at compile time in FDTD_common.hxx:1-76; the
runtime spec carries the same quantities plus the breast-imaging extensions.
"""
from __future__ import annotations

import ctypes as C

MODE_REFERENCE_GPU = 0
MODE_REFERENCE_CPU = 1
MODE_BREAST = 2
FP32 = 0
FP64 = 1
MAX_FREQS = 32


class Spec(C.Structure):
    _fields_ = [
        ("mode", C.c_int32),
        ("precision", C.c_int32),
        ("nx", C.c_int32),
        ("ny", C.c_int32),
        ("dx", C.c_double),
        ("dt", C.c_double),
        ("steps", C.c_int32),
        ("ncpml", C.c_int32),
        ("cpml_grading", C.c_double),
        ("cpml_sigma_max", C.c_double),
        ("cpml_kappa_max", C.c_double),
        ("cpml_alpha_max", C.c_double),
        ("cpml_alpha_min", C.c_double),
        ("tau", C.c_double),
        ("breast_radius", C.c_double),
        ("npatch", C.c_int32),
        ("n_excitations", C.c_int32),
        ("pw_tau", C.c_double),
        ("pw_t0", C.c_double),
        ("pw_l", C.c_double),
        ("pw_centred", C.c_int32),
        ("nan_clamp", C.c_int32),
        ("bg_eps_inf", C.c_double),
        ("bg_del_eps", C.c_double),
        ("bg_sigma", C.c_double),
        ("disc_radius", C.c_double),
        ("disc_eps_inf", C.c_double),
        ("disc_del_eps", C.c_double),
        ("disc_sigma", C.c_double),
        ("n_ellipses", C.c_int32),
        ("n_antennas", C.c_int32),
        ("n_tx", C.c_int32),
        ("antenna_radius", C.c_double),
        ("src_f0", C.c_double),
        ("src_tau", C.c_double),
        ("src_t0", C.c_double),
        ("src_amp", C.c_double),
        ("nf2ff_d", C.c_int32),
        ("nfreq", C.c_int32),
        ("freqs", C.c_double * MAX_FREQS),
        ("n_angles", C.c_int32),
        ("ff_norm", C.c_int32),
        ("misfit", C.c_int32),
        ("steps_per_launch", C.c_int32),
        ("cols_per_lane", C.c_int32),
        ("plain", C.c_int32),
        ("total_field", C.c_int32),
    ]

    def as_dict(self) -> dict:
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            if name == "freqs":
                v = [float(v[i]) for i in range(self.nfreq)]
            d[name] = v
        return d

    def copy(self, **changes) -> "Spec":
        s = Spec()
        C.memmove(C.byref(s), C.byref(self), C.sizeof(Spec))
        for k, v in changes.items():
            if k == "freqs":
                for i, f in enumerate(v):
                    s.freqs[i] = f
                s.nfreq = len(v)
            else:
                setattr(s, k, v)
        return s

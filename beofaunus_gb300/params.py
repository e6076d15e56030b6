"""ctypes mirror of ``fg_params`` (include/fg_params.h) plus builders for it.

One ``fg_params`` describes a Faunus system the way the reference's JSON input
does (``Space`` geometry, ``atomlist``, ``energy/nonbonded`` keys); see
include/fg_params.h for the reference provenance of every field.
"""
import ctypes

FG_MODEL_EWALD_WCA = 1
FG_MODEL_DH_LJ = 2
FG_MODEL_MULTIPOLE_RF = 3
FG_MODEL_EWALD_DIPOLE = 4
FG_EWALD_ION_ION = 1
FG_EWALD_ION_DIPOLE = 2
FG_EWALD_DIPOLE_DIPOLE = 4
FG_MAX_TYPES = 16

_D16 = ctypes.c_double * FG_MAX_TYPES


class FgParams(ctypes.Structure):
    _fields_ = [
        ("model", ctypes.c_int32),
        ("n_types", ctypes.c_int32),
        ("box", ctypes.c_double * 3),
        ("bjerrum", ctypes.c_double),
        ("type_charge", _D16),
        ("type_sigma", _D16),
        ("type_eps", _D16),
        ("type_dp", _D16),
        ("ewald_alpha", ctypes.c_double),
        ("ewald_cutoff", ctypes.c_double),
        ("ewald_cutoff_k", ctypes.c_double),
        ("ewald_debye_length", ctypes.c_double),
        ("ewald_eps_surf", ctypes.c_double),
        ("ewald_spherical_sum", ctypes.c_int32),
        ("ewald_update_frequency", ctypes.c_int32),
        ("dh_debye_length", ctypes.c_double),
        ("rf_cutoff", ctypes.c_double),
        ("rf_eps_rf", ctypes.c_double),
        ("rf_eps_r", ctypes.c_double),
        ("kT_scale", ctypes.c_double),
        ("use_cell_list", ctypes.c_int32),
        ("ewald_terms", ctypes.c_int32),
        ("ewald_dipole_quirk", ctypes.c_int32),
        ("ewald_isotropic_pbc", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 4),
    ]


def make_params(model, box, bjerrum, types, **kw):
    """Build an ``FgParams``.

    ``types`` is a list of dicts with keys q, sigma, eps (kT), dp (Angstrom),
    like the reference's ``atomlist`` entries after unit conversion.
    Remaining keyword arguments set fields by name (e.g. ewald_alpha=0.2).
    """
    p = FgParams()
    p.model = model
    p.n_types = len(types)
    if not 0 < len(types) <= FG_MAX_TYPES:
        raise ValueError("between 1 and %d atom types" % FG_MAX_TYPES)
    b = box if hasattr(box, "__len__") else (box, box, box)
    for d in range(3):
        p.box[d] = float(b[d])
    p.bjerrum = float(bjerrum)
    for i, t in enumerate(types):
        p.type_charge[i] = float(t["q"])
        p.type_sigma[i] = float(t["sigma"])
        p.type_eps[i] = float(t["eps"])
        p.type_dp[i] = float(t.get("dp", 0.0))
    p.ewald_spherical_sum = 1
    p.ewald_update_frequency = -1
    p.ewald_debye_length = 1e30
    p.kT_scale = 1.0
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p

"""ctypes / numpy mirrors of include/mic_types.h.

The marker record is byte-compatible with fvmic2d's ``Marker`` (fdcode.h:97-129,
216 bytes, cellX at offset 184); the material and boundary tables with
``Materials`` (fdcode.h:74-95) and ``BoundaryValues`` (fdcode.h:141-152).
"""
import ctypes

import numpy as np

MAXMAT = 8

MARKER_DTYPE = np.dtype(
    {
        "names": [
            "X", "Y", "VX", "VY", "Mat", "T", "Tdot",
            "sxx", "syy", "sxy", "eta", "mu", "rho", "rhodot", "p",
            "exx", "eyy", "exy", "Exx", "Eyy", "Exy", "Eii", "wxy",
            "cellX", "cellY", "cpu", "srr", "isYielding",
        ],
        "formats": [
            "<f8", "<f8", "<f8", "<f8", "<i4", "<f8", "<f8",
            "<f8", "<f8", "<f8", "<f8", "<f8", "<f8", "<f8", "<f8",
            "<f8", "<f8", "<f8", "<f8", "<f8", "<f8", "<f8", "<f8",
            "<i4", "<i4", "<i4", "<f8", "<i4",
        ],
        "offsets": [
            0, 8, 16, 24, 32, 40, 48,
            56, 64, 72, 80, 88, 96, 104, 112,
            120, 128, 136, 144, 152, 160, 168, 176,
            184, 188, 192, 200, 208,
        ],
        "itemsize": 216,
    }
)

# double-valued marker fields (name -> byte offset), used to address a field the way
# markerProjection.c:100-102 does (&markers[0].field with stride sizeof(Marker))
MARKER_F64_OFFSETS = {
    n: MARKER_DTYPE.fields[n][1]
    for n in MARKER_DTYPE.names
    if MARKER_DTYPE.fields[n][0] == np.dtype("<f8")
}


class Materials(ctypes.Structure):
    _fields_ = [
        ("nMaterials", ctypes.c_int32),
        ("materialEta", ctypes.c_double * MAXMAT),
        ("materialRho", ctypes.c_double * MAXMAT),
        ("materialkThermal", ctypes.c_double * MAXMAT),
        ("materialCp", ctypes.c_double * MAXMAT),
        ("materialAlpha", ctypes.c_double * MAXMAT),
        ("materialMu", ctypes.c_double * MAXMAT),
        ("materialFriction", ctypes.c_double * MAXMAT),
        ("materialCohesion", ctypes.c_double * MAXMAT),
        ("hasPlasticity", ctypes.c_int32 * MAXMAT),
        ("gamma", (ctypes.c_double * 2) * MAXMAT),
        ("C", (ctypes.c_double * 2) * MAXMAT),
        ("F", (ctypes.c_double * 2) * MAXMAT),
        ("hasEtaT", ctypes.c_int32 * MAXMAT),
        ("QonR", ctypes.c_double * MAXMAT),
        ("Tref", ctypes.c_double * MAXMAT),
    ]


class BCInfo(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32 * 3), ("value", ctypes.c_double * 3)]


class BCs(ctypes.Structure):
    _fields_ = [
        ("mechBCLeft", BCInfo),
        ("mechBCRight", BCInfo),
        ("mechBCTop", BCInfo),
        ("mechBCBottom", BCInfo),
    ]


class Options(ctypes.Structure):
    _fields_ = [
        ("etamin", ctypes.c_double),
        ("etamax", ctypes.c_double),
        ("fractionalEtamin", ctypes.c_double),
        ("subgridStressDiffusivity", ctypes.c_double),
        ("subgridTemperatureDiffusivity", ctypes.c_double),
        ("slabAngle", ctypes.c_double),
        ("decoupleThickness", ctypes.c_double),
        ("minDecoupleDepth", ctypes.c_double),
        ("maxDecoupleDepth", ctypes.c_double),
        ("decoupleEtaScaler", ctypes.c_double),
    ]


# nodal field ids (include/mic_types.h)
NF = {
    name: i
    for i, name in enumerate(
        [
            "rho", "rhodot", "etaS", "etaN", "thisT", "lastT", "kThermal", "Cp",
            "edotxx", "edotxy", "edotyy", "soxx", "soxy", "soyy", "dsxx", "dsyy", "dsxy",
            "muS", "muN", "vx", "vy", "p", "wxy", "srr", "eii", "sii", "heating",
        ]
    )
}
NF_COUNT = len(NF)

# fields written by projectMarkersNodesAll2 (markerProjection.c:11-68)
PROJECTED_FIELDS = ["rho", "rhodot", "etaN", "etaS", "muS", "muN", "kThermal", "lastT", "Cp", "soxx", "soyy", "soxy"]

ARITHMETIC, ARITHMETIC_LOCAL, HARMONIC = 0, 1, 2


class DensityOptions(ctypes.Structure):
    """mic_density_options: checkMarkerDensity settings (markers per cell at set-up, per
    quarter-cell bounds) and the subduction-benchmark parameters of the inflow markers it makes."""
    _fields_ = [("NMX", ctypes.c_int32), ("NMY", ctypes.c_int32), ("minMarkers", ctypes.c_int32),
                ("maxMarkers", ctypes.c_int32), ("slabAngle", ctypes.c_double), ("slabAge", ctypes.c_double),
                ("overridingPlateThickness", ctypes.c_double), ("rootThickness", ctypes.c_double),
                ("rootCenter", ctypes.c_double), ("rootWidth", ctypes.c_double)]


class SubductionOptions(ctypes.Structure):
    """mic_subduction_options: the Options fields the Stokes and thermal assemblies read
    (gravity, imposed slab velocity, slab / overriding-plate geometry, top thermal boundary)."""
    _fields_ = [("gx", ctypes.c_double), ("gy", ctypes.c_double), ("slabVelocity", ctypes.c_double),
                ("slabAngle", ctypes.c_double), ("slabAge", ctypes.c_double),
                ("overridingPlateThickness", ctypes.c_double), ("rootThickness", ctypes.c_double),
                ("rootCenter", ctypes.c_double), ("rootWidth", ctypes.c_double),
                ("thermalBCTopType", ctypes.c_int32), ("thermalBCTopValue", ctypes.c_double)]


class TimestepOptions(ctypes.Structure):
    """mic_timestep_options: one time step of main_subduction.c on the device"""
    _fields_ = [("dtMax", ctypes.c_double), ("displacementStepLimit", ctypes.c_double),
                ("maxTempChange", ctypes.c_double), ("maxNumPlasticity", ctypes.c_int32),
                ("shearHeating", ctypes.c_int32), ("firstStep", ctypes.c_int32), ("densityControl", ctypes.c_int32),
                ("density", DensityOptions), ("sub", SubductionOptions), ("adiabaticHeating", ctypes.c_int32),
                ("staticVelocity", ctypes.c_int32), ("thermalBCBottomValue", ctypes.c_double)]


class TimestepReport(ctypes.Structure):
    _fields_ = [("dt", ctypes.c_double), ("displacement_dt", ctypes.c_double), ("Kbond", ctypes.c_double),
                ("Kcont", ctypes.c_double), ("max_T", ctypes.c_double), ("residual", ctypes.c_double),
                ("max_temp_change", ctypes.c_double), ("max_abs_sxx", ctypes.c_double),
                ("plastic_iterations", ctypes.c_int32), ("is_yielding", ctypes.c_int32),
                ("converged", ctypes.c_int32), ("thermal_resolves", ctypes.c_int32), ("stopped", ctypes.c_int32),
                ("markers_added", ctypes.c_int64), ("markers_removed", ctypes.c_int64),
                ("nusselt", ctypes.c_double), ("vrms", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}

"""ctypes mirror of ``include/vacgpu.h``.

The structure below must stay field-for-field identical to ``vacgpu_params``
in the C header; ``tests/test_abi.py`` checks the size and offsets against the
compiled library (``vacgpu_params_size``/``vacgpu_params_offset``).
"""
import ctypes as C

MAXNW = 8
MAXB = 6
MAXEQPAR = 4
MAXSRCPAR = 8

PHYS_HD, PHYS_MHD = 0, 1
LIM_MINMOD, LIM_WOODWARD, LIM_SUPERBEE, LIM_VANLEER, LIM_ALBADA = range(5)
(BC_CONT, BC_PERIODIC, BC_SYMM, BC_ASYMM, BC_FIXED, BC_FIXED1, BC_CONT1, BC_GRAD1,
 BC_SYMM0, BC_SPECIAL) = range(10)
TVDLF, TVDLF1, TVDMU, TVDMU1 = 0, 1, 2, 3
ENTROPY_NUL, ENTROPY_HARTEN, ENTROPY_POWELL, ENTROPY_RATIO, ENTROPY_YEE = range(5)
LIMITED_ORIGINAL, LIMITED_PREVIOUS, LIMITED_PREDICTOR = range(3)
SPLIT_XYYX, SPLIT_XY = 0, 1
PREC_FP64, PREC_MIXED = 0, 1
SRC_NONE, SRC_GRAVITY = 0, 1

LIMITER_NAMES = {"minmod": LIM_MINMOD, "woodward": LIM_WOODWARD,
                 "superbee": LIM_SUPERBEE, "vanleer": LIM_VANLEER,
                 "albada": LIM_ALBADA}
TYPEFULL_NAMES = {"tvdlf": TVDLF, "tvdlf1": TVDLF1, "tvdmu": TVDMU,
                  "tvdmu1": TVDMU1}
ENTROPY_NAMES = {"nul": ENTROPY_NUL, "harten": ENTROPY_HARTEN,
                 "powell": ENTROPY_POWELL, "ratio": ENTROPY_RATIO,
                 "yee": ENTROPY_YEE}
BC_NAMES = {"cont": BC_CONT, "periodic": BC_PERIODIC, "symm": BC_SYMM,
            "asymm": BC_ASYMM, "fixed": BC_FIXED, "fixed1": BC_FIXED1,
            "cont1": BC_CONT1, "grad1": BC_GRAD1, "symm0": BC_SYMM0,
            "special": BC_SPECIAL}


class VacParams(C.Structure):
    _fields_ = [
        ("ndim", C.c_int),
        ("ndir", C.c_int),
        ("physics", C.c_int),
        ("nw", C.c_int),
        ("nx", C.c_int * 3),
        ("dixB", C.c_int),
        ("eqpar", C.c_double * MAXEQPAR),
        ("typefull", C.c_int),
        ("typelimiter", C.c_int * MAXNW),
        ("typelimited", C.c_int),
        ("dimsplit", C.c_int),
        ("typedimsplit", C.c_int),
        ("divbfix", C.c_int),
        ("sourceunsplit", C.c_int),
        ("courantpar", C.c_double),
        ("dtpar", C.c_double),
        ("smallpcoeff", C.c_double),
        ("smallp", C.c_double),
        ("slowsteps", C.c_int),
        ("dtcantgrow", C.c_int),
        ("tmaxexact", C.c_int),
        ("itmax", C.c_int),
        ("tmax", C.c_double),
        ("dtmin", C.c_double),
        ("typeB", (C.c_int * MAXNW) * MAXB),
        ("precision", C.c_int),
        ("smallfix", C.c_int),
        ("smallrho", C.c_double),
        ("smallrhocoeff", C.c_double),
        ("vacuumrho", C.c_double),
        ("useprimitive", C.c_int),
        ("compactres", C.c_int),
        ("dtdiffpar", C.c_double),
        ("typeentropy", C.c_int * MAXNW),
        ("entropycoef", C.c_double * MAXNW),
        ("divbwave", C.c_int),
    ]


def nw_of(physics, ndir):
    return 2 + 2 * ndir if physics == PHYS_MHD else 2 + ndir


def default_params(ndim, ndir, physics, nx, gamma=5.0 / 3.0):
    """par/DEFAULT values (par/DEFAULT:1-86 and the readparameters defaults,
    src/vacio.t:55-118) for a grid of ``nx`` mesh cells."""
    p = VacParams()
    p.ndim, p.ndir, p.physics = ndim, ndir, physics
    p.nw = nw_of(physics, ndir)
    for d in range(3):
        p.nx[d] = nx[d] if d < ndim else 1
    p.dixB = 2
    p.eqpar[0] = gamma
    p.typefull = TVDLF
    for iw in range(MAXNW):
        p.typelimiter[iw] = LIM_MINMOD
    p.typelimited = LIMITED_ORIGINAL
    p.dimsplit = 1
    p.typedimsplit = SPLIT_XYYX
    p.divbfix = 1
    p.sourceunsplit = 1
    p.courantpar = 0.8
    p.dtpar = -1.0
    p.smallpcoeff = 1.0e-6
    p.smallp = -1.0
    p.slowsteps = 0
    p.dtcantgrow = 0
    p.tmaxexact = 0
    p.itmax = 1000000
    p.tmax = 1.0e99
    p.dtmin = 1.0e-99
    for ib in range(MAXB):
        for iw in range(MAXNW):
            p.typeB[ib][iw] = BC_CONT
    p.precision = PREC_FP64
    p.smallfix = 0
    p.smallrho = -1.0
    p.smallrhocoeff = 1.0e-6
    p.vacuumrho = -1.0
    p.useprimitive = 0
    p.compactres = 0
    p.dtdiffpar = 0.5
    for il in range(MAXNW):
        p.typeentropy[il] = ENTROPY_NUL
        p.entropycoef[il] = default_entropycoef(physics, il)
    p.divbwave = 1
    return p


def default_entropycoef(physics, il):
    """physini's entropycoef of wave il (0-based): the default-real
    literals 0.2 and 0.4 of src/vacphys.mhd0.t:18-28 and
    src/vacphys.t.hd:21-29, i.e. single precision widened to double."""
    f02 = float(C.c_float(0.2).value)
    f04 = float(C.c_float(0.4).value)
    if physics == PHYS_MHD:
        if il < 4:        # fastRW, fastLW, slowRW, slowLW
            return f02
        if il in (6, 7):  # alfvRW, alfvLW
            return f04
        return -1.0
    return f02 if il < 2 else -1.0  # soundRW, soundLW


def set_all_bc(p, bc):
    for ib in range(MAXB):
        for iw in range(MAXNW):
            p.typeB[ib][iw] = bc


def set_all_limiters(p, lim):
    for iw in range(MAXNW):
        p.typelimiter[iw] = lim

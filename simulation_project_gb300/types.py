"""ctypes mirrors of the interface types in include/mps_types.h.

The field order and types follow the reference's DataType.h (radix/SPVSOLVER/
MultiGPUSolver/DataType.h:121-530); tests/test_types.py checks every offset against
offsets recorded from the reference header.
"""
import ctypes as C

import numpy as np

CCT_NOERR, CCT_FILEERR, CCT_PARAMERR, CCT_CALCERR, CCT_MEMERR, CCT_CUDAERR, CCT_ETCERR = range(7)
STATUS_NAMES = ["CCT_NOERR", "CCT_FILEERR", "CCT_PARAMERR", "CCT_CALCERR", "CCT_MEMERR", "CCT_CUDAERR", "CCT_ETCERR"]

TYPE_HEAVY_WEIGHT, TYPE_HEAVY_WEIGHT_FREE_SURFACE, TYPE_LIGHT_WEIGHT = 0, 1, 2
CELLMAXTRIANGLENUM = 100


class MpsError(RuntimeError):
    """An entry point returned a status other than CCT_NOERR."""

    def __init__(self, status: int, what: str = ""):
        name = STATUS_NAMES[status] if 0 <= status < len(STATUS_NAMES) else str(status)
        super().__init__(f"{what}: {name}" if what else name)
        self.status = status


def check(status: int, what: str = "") -> None:
    if status != CCT_NOERR:
        raise MpsError(status, what)


class Scalar3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class Integer3(C.Structure):
    _fields_ = [("x", C.c_int), ("y", C.c_int), ("z", C.c_int)]


class DragParameter(C.Structure):
    _fields_ = [
        ("DragID", C.c_int),
        ("DragToken", C.c_char),
        ("InputVelocityToken1", C.c_char),
        ("OutputVelocityToken2", C.c_char),
        ("CoefficientofInflueneRegion", C.c_float),
        ("VelocityIndex", C.c_float),
        ("VelocityExponential", C.c_float),
        ("VelocityDragPermiabilityConstant", C.c_float),
        ("TempIndex", C.c_float),
        ("TempExponential", C.c_float),
        ("TempDragPermiabilityConstant", C.c_float),
        ("ConstantVx", C.c_float),
        ("ConstantVy", C.c_float),
        ("ConstantVz", C.c_float),
        ("VelocityMagnitueFactor", C.c_float),
    ]


class CTriangleParameters(C.Structure):
    _fields_ = [
        ("Velocity", Scalar3),
        ("Temperature", C.c_float),
        ("LinearMovableOrNot", C.c_bool),
        ("LinearResetInterval", C.c_int),
        ("RotatingOrNot", C.c_bool),
        ("AngleOfRotationInDegree", C.c_float),
        ("RotationInRPM", C.c_float),
        ("RotationStartTime", C.c_float),
        ("TimeToReachRPM", C.c_float),
        ("CenterOfRotation", Scalar3),
        ("SecondPointOfRotation", Scalar3),
        ("InfluenceRegion", C.c_float),
        ("DirectionVector", Scalar3),
        ("NegativePressureCheck", C.c_bool),
        ("PressureGas", C.c_float),
        ("WallFrictionCoefficient", C.c_float),
        ("WallThermalResistivity", C.c_float),
        ("WallThermalConductivity", C.c_float),
        ("isDrag", C.c_bool),
        ("DragTriangleID", C.c_int),
    ]


class CTriangle(C.Structure):
    _fields_ = [("ModelIDNumber", C.c_int), ("Normal", Scalar3), ("Vertex", Scalar3 * 3)]


class CDistance(C.Structure):
    _fields_ = [("Magnitude", C.c_float), ("Direction", Scalar3)]


class CBox(C.Structure):
    _fields_ = [("m_MinBound", Scalar3), ("m_MaxBound", Scalar3)]


class CGridBox(C.Structure):
    _fields_ = [
        ("m_BufferedZone", CBox),
        ("m_ComputeZone", CBox),
        ("m_PressureZone", CBox),
        ("m_ParentZone", CBox),
        ("m_GridSize", Integer3),
        ("m_CellSize", C.c_float),
    ]

    @property
    def cell_num(self) -> int:
        g = self.m_GridSize
        return g.x * g.y * g.z


class CCell(C.Structure):
    _fields_ = [("m_TriangleNum", C.c_uint), ("m_TriangleID", C.c_int * CELLMAXTRIANGLENUM)]


_CPARAM_FIELDS = [
    ("Dimension", C.c_int),
    ("GravityConstant", Scalar3),
    ("Density", C.c_float),
    ("ConstantParticleDensity", C.c_float),
    ("SurfaceTensionCoefficient", C.c_float),
    ("InitialParticleDistance", C.c_float),
    ("FreeSurfaceThreshold", C.c_float),
    ("GradientInfluenceRadiusCoefficient", C.c_float),
    ("LaplacianInfluenceRadiusCoefficient", C.c_float),
    ("TemperatureInfluenceRadiusCoefficient", C.c_float),
    ("FruidInitializeialTemperature", C.c_float),
    ("WallInitializeialTemperature", C.c_float),
    ("FruidThermalResistance", C.c_float),
    ("WallThermalResistance", C.c_float),
    ("FruidThermalConductivity", C.c_float),
    ("WallThermalConductivity", C.c_float),
    ("FruidSpecificHeat", C.c_float),
    ("FruidDensity", C.c_float),
    ("Dt", C.c_float),
    ("AnalysisStep", C.c_int),
    ("ThermalStep", C.c_int),
    ("NegativeCalculationStep", C.c_int),
    ("OutputStep", C.c_int),
    ("LambdaID", C.c_int),
    ("SORJacobianRelaxationCoefficient", C.c_float),
    ("SORLoopMax", C.c_int),
    ("SORConvergenceConstant", C.c_float),
    ("bUpdateTemperature", C.c_bool),
    ("LambdaValue", C.c_float),
    ("CellSize", Scalar3),
    ("MvVelocity", Scalar3),
    ("CourantNumber", C.c_float),
    ("ViscosityUpdateParameterA", C.c_float),
    ("ViscosityUpdateParameterB", C.c_float),
    ("MaxWallTemperature", C.c_float),
    ("MinWallTemperature", C.c_float),
    ("OffSet", C.c_float),
    ("ParticleGenerationStep", C.c_int),
    ("TotalGenerationStep", C.c_int),
    ("Alpha", C.c_float),
    ("AlphaLightWeight", C.c_float),
    ("MaxNeighborhoodNum", C.c_int),
    ("bExplicitCollisonCheck", C.c_bool),
    ("bExplicitCollisionOut", C.c_bool),
    ("bImplicitCollisonCheck", C.c_bool),
    ("CollisionCheckCoefficient", C.c_float),
    ("MinDistanceCoefficient", C.c_float),
    ("bFreeSurfacePressureUpdate", C.c_bool),
    ("BasePressure", C.c_float),
    ("MaxPressure", C.c_float),
    ("Time1", C.c_float),
    ("TriggerStep", C.c_int),
    ("EndStep", C.c_int),
    ("AnalysisArea", C.c_float),
    ("bExplicitOut", C.c_bool),
    ("WallFrictionCoeffieicnt", C.c_float),
    ("DragCoefficient", C.c_float),
    ("bTwoPhase", C.c_bool),
    ("StopWallStep", C.c_int),
    ("Tolerance", C.c_float),
    ("ImplicitSurfaceThreshold", C.c_float),
    ("bCGSolver", C.c_bool),
    ("bUpdateInnerPressure", C.c_bool),
    ("SurfaceInfluenceRadiusCoefficient", C.c_float),
    ("SurfaceThreshold", C.c_float),
    ("GradientForce", C.c_float),
    ("StartStep", C.c_int),
    ("InitialForce", C.c_float),
    ("VelocityThreshold", C.c_float),
    ("bExplicitPressure", C.c_bool),
    ("SonicVelocity", C.c_float),
    ("ArtificialPressure", C.c_float),
    ("r_coeff", C.c_float),
    ("bImplicitVelocity", C.c_bool),
    ("bNJPCGSolver", C.c_bool),
    ("PressureMax", C.c_float),
    ("RLimitCoefficient", C.c_float),
    ("bTurbulance", C.c_bool),
    ("SmagorinskyConstant", C.c_float),
    ("FilterWidth", C.c_float),
    ("TurbulanViscosityRatio", C.c_float),
    ("Cnue", C.c_float),
    ("Cepsilon", C.c_float),
    ("TurbulanceIntensity", C.c_float),
    ("bNegativePressure", C.c_bool),
    ("InitialTimeForZeroAngle", C.c_float),
    ("FinalTimeToReachAngle", C.c_float),
    ("ConstantCheckStep", C.c_int),
]


class CParameter(C.Structure):
    _fields_ = _CPARAM_FIELDS


def s3(v) -> Scalar3:
    return Scalar3(float(v[0]), float(v[1]), float(v[2]))


def grid_box(compute_min, compute_max, param: CParameter) -> CGridBox:
    """Grid geometry of CCellSet::SetComputeZone (CGPUCellSet.cpp:109-152), in float:
    cell = l0*max(re_lap, re_grad); buffered zone = compute zone -/+ 2 cells;
    grid size = ceil(extent/cell + 4)."""
    f = np.float32
    mx = max(f(param.LaplacianInfluenceRadiusCoefficient), f(param.GradientInfluenceRadiusCoefficient))
    r = f(f(param.InitialParticleDistance) * f(mx))
    lo = np.array(compute_min, dtype=np.float32)
    hi = np.array(compute_max, dtype=np.float32)
    b = CGridBox()
    b.m_ComputeZone = CBox(s3(lo), s3(hi))
    b.m_ParentZone = CBox(s3(lo), s3(hi))
    b.m_PressureZone = CBox(s3(lo - r), s3(hi + r))
    b.m_BufferedZone = CBox(s3(lo - f(2) * r), s3(hi + f(2) * r))
    b.m_CellSize = float(r)
    gs = [int(np.ceil(f(f(hi[a] - lo[a]) / r) + f(4))) for a in range(3)]
    b.m_GridSize = Integer3(*gs)
    return b


def as_ptr(a: np.ndarray, ctype=C.c_void_p):
    """Pointer to a contiguous numpy array (None for None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return a.ctypes.data_as(ctype)


def structs_from_array(arr: np.ndarray, ctype):
    return (ctype * (arr.nbytes // C.sizeof(ctype))).from_buffer(arr)


# numpy dtypes with the same layout as the structs (for bulk arrays)
TRIANGLE_DTYPE = np.dtype([("ModelIDNumber", "<i4"), ("Normal", "<f4", 3), ("Vertex", "<f4", (3, 3))])
DISTANCE_DTYPE = np.dtype([("Magnitude", "<f4"), ("Direction", "<f4", 3)])
CELL_DTYPE = np.dtype([("m_TriangleNum", "<u4"), ("m_TriangleID", "<i4", CELLMAXTRIANGLENUM)])
assert TRIANGLE_DTYPE.itemsize == C.sizeof(CTriangle)
assert DISTANCE_DTYPE.itemsize == C.sizeof(CDistance)
assert CELL_DTYPE.itemsize == C.sizeof(CCell)

CParticle_size = 52   # sizeof(CParticle) (DataType.h:220-240)


class CParticle(C.Structure):
    """One particle record of the reference (DataType.h:220-240): the particle-file and
    bucket format."""
    _fields_ = [("ID", C.c_int), ("Position", Scalar3), ("Velocity", Scalar3), ("Pressure", C.c_float),
                ("Density", C.c_float), ("Temperature", C.c_float), ("KineticViscosity", C.c_float),
                ("SolidPhaseRate", C.c_float), ("Type", C.c_int)]

/*
 * mps_types.h - data types shared by every entry point of the GB300 MPS hot path.
 *
 * These are the interface types of the reference solver's kernel boundary.  Their
 * binary layout (field order, field types, natural alignment) is the one the
 * reference passes through its launcher API and constant-memory bindings, so a
 * caller written against the reference can hand the same structs to this library:
 *
 *   CCTStatusType          radix/SPVSOLVER/MultiGPUSolver/DataType.h:77-86
 *   ParticleType           DataType.h:88-105
 *   DragParameter          DataType.h:121-145
 *   CTriangleParameters    DataType.h:147-178
 *   CTriangle              DataType.h:180-203
 *   CDragTriangle          DataType.h:205-218
 *   CParticle              DataType.h:220-240
 *   CDistance, CBox, CGridBox   DataType.h:260-278
 *   CCell (+ CELLMAXTRIANGLENUM) DataType.h:308-315
 *   CParameter             DataType.h:318-530
 *
 * Scalar is float, as in every build of the reference (DOUBLE is never defined).
 * The header is plain C and also compiles as C++ and CUDA.
 */
#ifndef MPS_TYPES_H
#define MPS_TYPES_H

#include <stdint.h>
#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef float Scalar;
typedef int   Integer;

typedef struct MpsScalar3 { float x, y, z; } Scalar3;
typedef struct MpsInteger3 { int x, y, z; } Integer3;

/* Status codes returned by every entry point (0 = success). */
typedef enum CCTStatusType {
    CCT_NOERR = 0,
    CCT_FILEERR = 1,
    CCT_PARAMERR = 2,
    CCT_CALCERR = 3,
    CCT_MEMERR = 4,
    CCT_CUDAERR = 5,
    CCT_ETCERR = 6
} CCTStatusType;

typedef enum ParticleType {
    TYPE_HEAVY_WEIGHT = 0,
    TYPE_HEAVY_WEIGHT_FREE_SURFACE = 1,
    TYPE_LIGHT_WEIGHT = 2
} ParticleType;

/* Per drag model parameters ("D/DE/DC/DF" model lines of the configuration file). */
typedef struct DragParameter {
    Integer DragID;
    char DragToken;             /* 'E' exponential, 'C' constant velocity, 'F' velocity factor */
    char InputVelocityToken1;   /* 'V' velocity, 'T' temperature, 'B' both */
    char OutputVelocityToken2;
    Scalar CoefficientofInflueneRegion;   /* influence radius in units of l0 */
    float VelocityIndex;
    float VelocityExponential;
    float VelocityDragPermiabilityConstant;
    float TempIndex;
    float TempExponential;
    float TempDragPermiabilityConstant;
    float ConstantVx;
    float ConstantVy;
    float ConstantVz;
    float VelocityMagnitueFactor;
} DragParameter;

/* Per STL model motion / wall parameters. */
typedef struct CTriangleParameters {
    Scalar3 Velocity;
    Scalar Temperature;
    bool LinearMovableOrNot;
    Integer LinearResetInterval;
    bool RotatingOrNot;
    Scalar AngleOfRotationInDegree;   /* per-step increment: RPM * dt * 6 */
    Scalar RotationInRPM;
    Scalar RotationStartTime;
    Scalar TimeToReachRPM;
    Scalar3 CenterOfRotation;
    Scalar3 SecondPointOfRotation;
    Scalar InfluenceRegion;
    Scalar3 DirectionVector;
    bool NegativePressureCheck;
    Scalar PressureGas;
    Scalar WallFrictionCoefficient;
    Scalar WallThermalResistivity;
    Scalar WallThermalConductivity;
    bool isDrag;
    Integer DragTriangleID;
} CTriangleParameters;

/* One wall triangle: owning model, unit normal, three vertices (52 bytes). */
typedef struct CTriangle {
    Integer ModelIDNumber;
    Scalar3 Normal;
    Scalar3 Vertex[3];
} CTriangle;

typedef struct CDragTriangle {
    Scalar3 Normal;
    Scalar3 Vertex[3];
    Scalar DragLength;
    Integer StartStep01;
    Integer StartStep02;
    Integer EndStep;
    Scalar3 InitialAcc;
    Scalar3 GradAcc;
    Integer ID;
} CDragTriangle;

typedef struct CParticle {
    Integer ID;
    Scalar3 Position;
    Scalar3 Velocity;
    Scalar Pressure;
    Scalar Density;
    Scalar Temperature;
    Scalar KineticViscosity;
    Scalar SolidPhaseRate;
    ParticleType Type;
} CParticle;

/* Nearest-wall record: distance magnitude and the vector from the wall to the particle. */
typedef struct CDistance {
    Scalar Magnitude;
    Scalar3 Direction;
} CDistance;

typedef struct CBox {
    Scalar3 m_MinBound;
    Scalar3 m_MaxBound;
} CBox;

/* Uniform grid: cell (i,j,k) of a position p is (int)((p - BufferedZone.min) / CellSize);
 * its key is (GridSize.y*GridSize.z)*i + GridSize.z*j + k. */
typedef struct CGridBox {
    CBox m_BufferedZone;
    CBox m_ComputeZone;
    CBox m_PressureZone;
    CBox m_ParentZone;
    Integer3 m_GridSize;
    Scalar m_CellSize;
} CGridBox;

#define CELLMAXTRIANGLENUM 100
/* Fixed-capacity per-cell triangle list of the reference layout (404 bytes per cell). */
typedef struct CCell {
    unsigned int m_TriangleNum;
    Integer m_TriangleID[CELLMAXTRIANGLENUM];
} CCell;

/* Solver parameters, in the order of the positional parameter file. */
typedef struct CParameter {
    int Dimension;
    Scalar3 GravityConstant;
    Scalar Density;                         /* fluid density rho */
    Scalar ConstantParticleDensity;         /* n0 */
    Scalar SurfaceTensionCoefficient;
    Scalar InitialParticleDistance;         /* l0 */
    Scalar FreeSurfaceThreshold;            /* beta */
    Scalar GradientInfluenceRadiusCoefficient;
    Scalar LaplacianInfluenceRadiusCoefficient;
    Scalar TemperatureInfluenceRadiusCoefficient;
    Scalar FruidInitializeialTemperature;
    Scalar WallInitializeialTemperature;
    Scalar FruidThermalResistance;
    Scalar WallThermalResistance;
    Scalar FruidThermalConductivity;
    Scalar WallThermalConductivity;
    Scalar FruidSpecificHeat;
    Scalar FruidDensity;
    Scalar Dt;
    Integer AnalysisStep;
    Integer ThermalStep;
    Integer NegativeCalculationStep;
    Integer OutputStep;
    Integer LambdaID;
    Scalar SORJacobianRelaxationCoefficient;
    Integer SORLoopMax;
    Scalar SORConvergenceConstant;
    bool bUpdateTemperature;
    Scalar LambdaValue;
    Scalar3 CellSize;
    Scalar3 MvVelocity;
    Scalar CourantNumber;
    Scalar ViscosityUpdateParameterA;
    Scalar ViscosityUpdateParameterB;
    Scalar MaxWallTemperature;
    Scalar MinWallTemperature;
    Scalar OffSet;
    Integer ParticleGenerationStep;
    Integer TotalGenerationStep;
    Scalar Alpha;
    Scalar AlphaLightWeight;
    Integer MaxNeighborhoodNum;
    bool bExplicitCollisonCheck;
    bool bExplicitCollisionOut;
    bool bImplicitCollisonCheck;
    Scalar CollisionCheckCoefficient;
    Scalar MinDistanceCoefficient;
    bool bFreeSurfacePressureUpdate;
    Scalar BasePressure;
    Scalar MaxPressure;
    Scalar Time1;
    Integer TriggerStep;
    Integer EndStep;
    Scalar AnalysisArea;
    bool bExplicitOut;
    Scalar WallFrictionCoeffieicnt;
    Scalar DragCoefficient;
    bool bTwoPhase;
    Integer StopWallStep;
    Scalar Tolerance;
    Scalar ImplicitSurfaceThreshold;
    bool bCGSolver;
    bool bUpdateInnerPressure;
    Scalar SurfaceInfluenceRadiusCoefficient;
    Scalar SurfaceThreshold;
    Scalar GradientForce;
    Integer StartStep;
    Scalar InitialForce;
    Scalar VelocityThreshold;
    bool bExplicitPressure;
    Scalar SonicVelocity;
    Scalar ArtificialPressure;
    Scalar r_coeff;
    bool bImplicitVelocity;
    bool bNJPCGSolver;
    Scalar PressureMax;
    Scalar RLimitCoefficient;
    bool bTurbulance;
    Scalar SmagorinskyConstant;
    Scalar FilterWidth;
    Scalar TurbulanViscosityRatio;
    Scalar Cnue;
    Scalar Cepsilon;
    Scalar TurbulanceIntensity;
    bool bNegativePressure;
    Scalar InitialTimeForZeroAngle;
    Scalar FinalTimeToReachAngle;
    Integer ConstantCheckStep;
} CParameter;

#ifdef __cplusplus
}
#endif

#endif /* MPS_TYPES_H */

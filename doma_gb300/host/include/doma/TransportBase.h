// TransportBase.h -- enumerations of DOMA's public interface, kept with the
// same names and values so code written against DOMA compiles unchanged
// (DOMA include/TransportBase.h:1-62; "CertesianFaceSide" keeps DOMA's spelling).
#pragma once

enum class CertesianAxis { X = 0u, Y = 1u, Z = 2u };

enum class CertesianFaceSide { Right = 0u, Left = 1u, Front = 2u, Back = 3u, Top = 4u, Bottom = 5u };

enum class Octant { PPP = 0u, PPM = 1u, PMP = 2u, PMM = 3u, MPP = 4u, MPM = 5u, MMP = 6u, MMM = 7u };

enum class BoundaryCondition { Vacuum = 0u, Reflective = 1u };

enum class RunMode { FixedSrc = 0u, Eigen = 1u, Transient = 2u };

enum class EquationType { DD = 0u, TW_DD = 1u };

enum class TransientIC { Zero = 0u, SteadyState = 1u };

enum class StepType { Insert = 0u, Remove = 1u, Both = 2u };

// GPU-only choice, not part of DOMA: arithmetic of the sweep.
enum class SweepPrecision { FP64 = 0u, FP32 = 1u };

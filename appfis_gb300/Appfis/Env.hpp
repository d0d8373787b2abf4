/*
 * Env.hpp — API macros, enums and the execution flag of the GB300 APPFIS engine.
 *
 * Same names and meanings as the reference (Appfis/Env.hpp:16-32): PARALLEL marks a user
 * Stencil overload as device code, EXEC_SPACE marks Array accessors as host+device code, and
 * STENCIL is the name every user functor overload carries.  This engine always runs the sweeps
 * on the GPU, so an application must be compiled with nvcc (-x cu).
 */
#ifndef APPFIS_GB_ENV_HPP
#define APPFIS_GB_ENV_HPP

#if !defined(__CUDACC__)
#error "The GB300 APPFIS engine runs every stencil on the GPU: compile the application with nvcc (-x cu)."
#endif

#include <cuda_runtime.h>

namespace APPFIS
{

#define PARALLEL __device__
#define EXEC_SPACE __host__ __device__
#define STENCIL Stencil

	enum AXIS { X, Y, Z };
	enum DIMENSION { DIM_1D = 1, DIM_2D = 2, DIM_3D = 3 };
	enum DIRECTION { LEFT, RIGHT, UP, DOWN, FRONT, BACK };
	enum GRID_TYPE { SINGLE, DUAL, FLAT };
	enum REDUCTION { MAX, MIN, SUM };

	// True between InitializeExecution and FinalizeExecution: GetSubGrid() then hands out
	// descriptors of the device buffers instead of the host arrays.
	inline bool& ExecutionFlag()
	{
		static bool flag = false;
		return flag;
	}

}

#endif

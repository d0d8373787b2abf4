/*
 * Common.hpp — the run context and its getters.
 *
 * The reference keeps an MPI Cartesian topology, the OpenMP thread count and one CUDA stream
 * in a singleton (Appfis/Topology.hpp:104-210) behind free functions (Appfis/Common.hpp:19-226).
 * On one GB300 the decomposition is a single rank: every block count is 1, coordinates are 0,
 * a periodic axis is its own neighbour and a non-periodic one has none.  The context keeps the
 * ghost width, periodicity and the engine's CUDA stream.
 */
#ifndef APPFIS_GB_COMMON_HPP
#define APPFIS_GB_COMMON_HPP

#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>

#include "Env.hpp"
#include "Attribute.hpp"
#include "appfis_gb.h"

namespace APPFIS
{

	const int PROC_NULL = -2;

	struct Context
	{
		int nDim = 0;
		int pDim = 0;
		int ghostLayer = 1;
		bool periodic = false;
		bool overlap = false;
		int threads = 1;
		int blocks[3] = { 1, 1, 1 };
		int coords[3] = { 0, 0, 0 };
		int neighbours[6] = { PROC_NULL, PROC_NULL, PROC_NULL, PROC_NULL, PROC_NULL, PROC_NULL };
		cudaStream_t stream = 0;
		bool initialized = false;
		// set once a Config is routed to a hand-written kernel (Fast.hpp): run the sweeps it
		// deferred / also free its buffers
		void (*flushFast)() = nullptr;
		void (*releaseFast)() = nullptr;

		static Context& Get()
		{
			static Context ctx;
			return ctx;
		}
	};

	// Aborts with the library's message when an engine call fails (the reference prints to
	// std::cerr and exits on setup errors; here every engine status is checked).
	inline void Check(int status, const char* what)
	{
		if (status != APPFIS_GB_OK)
		{
			std::cerr << "APPFIS engine: " << what << " failed: " << appfis_gb_last_error() << std::endl;
			std::exit(EXIT_FAILURE);
		}
	}

	inline void CheckCuda(cudaError_t e, const char* what)
	{
		if (e != cudaSuccess)
		{
			std::cerr << "APPFIS engine: " << what << " failed: " << cudaGetErrorString(e) << std::endl;
			std::exit(EXIT_FAILURE);
		}
	}

	inline void Initialize(int argc, char* argv[], int dataDim, int partitionDim, Attribute attribute = ATTRIBUTE)
	{
		(void)argc;
		(void)argv;
		if (partitionDim > dataDim)
		{
			std::cerr << "Initialization failed. Partition dimension (" << partitionDim
				<< ") can not be larger than data dimension (" << dataDim << ")." << std::endl;
			std::exit(EXIT_FAILURE);
		}
		Context& c = Context::Get();
		c.nDim = dataDim;
		c.pDim = partitionDim;
		c.ghostLayer = attribute.ghostLayer;
		c.periodic = attribute.periodic;
		c.overlap = attribute.overlap;
		c.threads = attribute.threads;
		for (int f = 0; f < 6; f++) c.neighbours[f] = c.periodic ? 0 : PROC_NULL;
		int dev = 0;
		CheckCuda(cudaGetDevice(&dev), "cudaGetDevice");
		CheckCuda(cudaSetDevice(dev), "cudaSetDevice");
		if (!c.stream) CheckCuda(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking), "cudaStreamCreate");
		c.initialized = true;
		std::string s = "Process Dims:";
		for (int i = 0; i < dataDim; i++) s += " 1";
		std::cout << s << std::endl;
	}

	inline void Finalize()
	{
		Context& c = Context::Get();
		if (c.releaseFast) c.releaseFast();
		if (c.stream) cudaStreamSynchronize(c.stream);
	}

	inline int GetRank() { return 0; }
	inline int GetMasterRank() { return 0; }
	inline int GetRankCount() { return 1; }
	inline int GetNeighbourCount() { return Context::Get().nDim * 2; }
	inline int GetDimCount() { return Context::Get().nDim; }
	inline int GetPartitionDim() { return Context::Get().pDim; }
	inline int GetGhostLayer() { return Context::Get().ghostLayer; }
	inline bool IsMaster() { return true; }
	inline bool IsOverlap() { return Context::Get().overlap; }
	inline bool IsPeriodic() { return Context::Get().periodic; }
	inline int* GetBlocks() { return Context::Get().blocks; }
	inline int* GetCoords() { return Context::Get().coords; }
	inline int GetNeighboursRank(int face) { return Context::Get().neighbours[face]; }
	inline cudaStream_t& GetCudaStream() { return Context::Get().stream; }

	inline void SetMasterRank(int master)
	{
		if (master != 0) std::cerr << "Setting master rank to " << master << " has failed. Default value 0." << std::endl;
	}

	// Local (ghost-padded) dims of the single rank: full dims + 2*ghost (Appfis/Common.hpp:197-226
	// with one block per axis).
	inline void GetLocalPartitionDims(int nDim, int* fullDataDims, int* subDataDims)
	{
		const int g = GetGhostLayer();
		for (int i = 0; i < nDim; i++)
		{
			if (fullDataDims[i] < 2 * g)
			{
				std::cerr << "Subgrid Data dimension should be at least: " << (2 * g) << ". Found: " << fullDataDims[i] << std::endl;
				std::exit(EXIT_FAILURE);
			}
			subDataDims[i] = fullDataDims[i] + 2 * g;
		}
	}

}

#endif

/*
 * Runtime.hpp — InitializeExecution / FinalizeExecution / Execute{1,2,3}D / Execute*DReduce /
 * HaloExchange of the GB300 APPFIS engine (reference: Appfis/Runtime.hpp:23-255 dispatch,
 * Appfis/Runtime_CUDA.hpp:231-740 GPU path).
 *
 * Execute*D(config, args...) launches one generic kernel over the Config box that calls the
 * user's Stencil(i[, j[, k]], args...) per point, exactly like the reference's Kernel{1,2,3}D
 * (Runtime_CUDA.hpp:1201-1246), with these differences:
 *   - every Array<T>* argument travels by value (pointer + dims) and is rebuilt in registers,
 *     so Get/Set do no dependent load of a dims pointer; when all array arguments share one
 *     shape (checked on the host per launch) the views are rebuilt from a single copy of it,
 *     so a point's linear index is formed once for all arrays (Himeno's 14 arrays: 66 -> 77
 *     GLUP/s on GB300, the radius-4 star 139 -> 147); boxes whose rows are not a multiple of 32
 *     wide, and launches without the march below, number the points of each (x, y) plane
 *     consecutively, so warps do not straddle a mostly idle row end (Himeno's 129-wide rows:
 *     77 -> 88; Triton's FP64 functors 2.72 -> 3.14 with the 2-D march limited to two arrays);
 *   - blocks are 32 wide in x (coalesced rows) for every dimensionality;
 *   - after the sweep, the grids named by GridsToUpdate get their periodic ghosts refreshed on
 *     the device (no pack / host copy / MPI round trip) and are swapped; with one rank and no
 *     periodic axis there is nothing to exchange, as in the reference.
 * Reductions run on the device in one deterministic launch (appfis_gb_reduce) and return the
 * value to the host like the reference's Execute*DReduceGPU (Runtime_CUDA.hpp:554-740), seeds
 * included (MAX starts from numeric_limits<T>::min()); the input grid is never overwritten.
 * The reference's GPU 1-D executor swaps the updated grids twice (Runtime_CUDA.hpp:295-296), a
 * net no-op; here every executor swaps once, like the reference's CPU path (Runtime.hpp:318-319).
 */
#ifndef APPFIS_GB_RUNTIME_HPP
#define APPFIS_GB_RUNTIME_HPP

#include <cstdlib>
#include <iostream>
#include <type_traits>

#include "Config.hpp"
#include "Fast.hpp"
#include "Grid.hpp"

namespace APPFIS
{

	namespace detail
	{
		inline int gb_launch_status()
		{
			const cudaError_t e = cudaGetLastError();
			if (e == cudaSuccess) return APPFIS_GB_OK;
			std::cerr << "APPFIS engine: " << cudaGetErrorString(e) << std::endl;
			return APPFIS_GB_ECUDA;
		}

		// Host -> kernel argument conversion: Array<U>* becomes a by-value view of device memory.
		template<class A>
		struct KArg
		{
			typedef A type;
			static A to(A a) { return a; }
		};

		template<class U>
		struct KArg<Array<U>*>
		{
			typedef ArrayArg<U> type;
			static ArrayArg<U> to(Array<U>* a)
			{
				if (a != nullptr && a->IsDeviceView()) return a->Arg();  // a grid's device view: no driver query
				cudaPointerAttributes attr;
				if (a == nullptr || a->GetData() == nullptr || cudaPointerGetAttributes(&attr, a->GetData()) != cudaSuccess ||
					attr.type != cudaMemoryTypeDevice)
				{
					cudaGetLastError();
					std::cerr << "APPFIS engine: an Array passed to Execute*D is not on the device; pass grid.GetSubGrid() "
						"after InitializeExecution(grid)." << std::endl;
					std::exit(EXIT_FAILURE);
				}
				return a->Arg();
			}
		};

		// Kernel side: scalars pass through, array views are rebuilt as local Array objects.
		template<class A>
		struct Holder
		{
			A v;
			__device__ explicit Holder(const A& a) : v(a) {}
			__device__ A get() const { return v; }
		};

		template<class U>
		struct Holder<ArrayArg<U> >
		{
			Array<U> a;
			__device__ explicit Holder(const ArrayArg<U>& g) : a(g) {}
			__device__ Array<U>* get() { return &a; }
		};

		template<class... A>
		__global__ void Functor1D(int x0, int x1, A... args)
		{
			const int i = x0 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
			if (i < x1) STENCIL(i, Holder<A>(args).get()...);
		}

		// Rows (2-D) or planes (3-D) per thread: a thread calls the functor for MARCH consecutive
		// points along its slowest axis, so the neighbour values of one call are in L1 for the next.
		// Every point of the box is still visited exactly once, in no particular order.  The march
		// pays only for functors over a few fields (measured on GB300: the radius-4 star over 2
		// arrays 107 -> 139 GLUP/s; Himeno over 14 arrays 68 -> 48, its loads in flight are what
		// count), so functors taking more than MARCH_MAX_ARRAYS arrays keep one point per thread.
		// In 2-D the march pays only for functors over one or two fields (GameOfLife); Triton's
		// pointwise dt and 5-point wet/dry functors over 4 arrays ran 8% faster without it.
		// Depth: 4 rows in 2-D (GameOfLife 319 GLUP/s; 2 rows: 290, 8 rows: 315), 8 planes in
		// 3-D (the star 147.7; 4 planes: 146.0, 2 planes: 135).
		constexpr int MARCH = 4, MARCH_3D = 8, MARCH_MAX_ARRAYS = 4, MARCH_MAX_ARRAYS_2D = 2;

		template<class A> struct IsArrayArg { static const int value = 0; };
		template<class U> struct IsArrayArg<ArrayArg<U> > { static const int value = 1; };
		template<class... A> struct ArrayCount { static const int value = 0; };
		template<class H, class... R> struct ArrayCount<H, R...>
		{
			static const int value = IsArrayArg<H>::value + ArrayCount<R...>::value;
		};

		// Shape of every array argument of a launch, when they all agree (checked on the host):
		// the uniform kernels rebuild each view from this one copy, so the compiler sees a single
		// set of dims and forms a point's linear index once for all arrays instead of once per
		// array.  The functor, its arguments and the visit order are the same as the other kernels'.
		struct Shape
		{
			int nDim, size;
			int d[3];
		};

		inline void Agree(Shape&, bool&, int&) {}

		template<class H, class... R>
		void Agree(Shape& s, bool& ok, int& n, const H&, const R&... r) { Agree(s, ok, n, r...); }

		template<class U, class... R>
		void Agree(Shape& s, bool& ok, int& n, Array<U>* const& a, const R&... r)
		{
			if (a == nullptr)
				ok = false;
			else if (n++ == 0)
			{
				s.nDim = a->GetDimCount();
				s.size = a->GetSize();
				for (int k = 0; k < 3; k++) s.d[k] = a->GetDim(k);
			}
			else if (a->GetDimCount() != s.nDim || a->GetSize() != s.size || a->GetDim(0) != s.d[0] || a->GetDim(1) != s.d[1] ||
				a->GetDim(2) != s.d[2])
				ok = false;
			Agree(s, ok, n, r...);
		}

		// True when the launch has array arguments and all of them share one shape (into s).
		template<class... TArgs>
		bool UniformShape(Shape& s, const TArgs&... args)
		{
			bool ok = true;
			int n = 0;
			Agree(s, ok, n, args...);
			return ok && n > 0;
		}

		template<class A>
		struct HolderU
		{
			A v;
			__device__ HolderU(const A& a, const Shape&) : v(a) {}
			__device__ A get() const { return v; }
		};

		template<class U>
		struct HolderU<ArrayArg<U> >
		{
			Array<U> a;
			__device__ HolderU(const ArrayArg<U>& g, const Shape& s) : a(g.data, s.nDim, s.size, s.d) {}
			__device__ Array<U>* get() { return &a; }
		};

		template<int M, class... A>
		__global__ void Functor2DU(int x0, int x1, int y0, int y1, Shape s, A... args)
		{
			const int i = x0 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
			const int jb = y0 + (int)(blockIdx.y * blockDim.y + threadIdx.y) * M;
			if (i >= x1) return;
			for (int j = jb; j < jb + M && j < y1; j++) STENCIL(i, j, HolderU<A>(args, s).get()...);
		}

		template<int M, class... A>
		__global__ void Functor3DU(int x0, int x1, int y0, int y1, int z0, int z1, Shape s, A... args)
		{
			const int i = x0 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
			const int j = y0 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
			const int kb = z0 + (int)(blockIdx.z * blockDim.z + threadIdx.z) * M;
			if (i >= x1 || j >= y1) return;
			for (int k = kb; k < kb + M && k < z1; k++) STENCIL(i, j, k, HolderU<A>(args, s).get()...);
		}

		// Division by a launch-constant d > 0 as a multiply and shift: q = (n * m) >> k with
		// k = 31 + ceil(log2 d), m = ceil(2^k / d), exact for every n < 2^31 (the error term
		// n * (m*d - 2^k) stays below 2^k), and n * m < 2^64.
		struct Div
		{
			unsigned long long m;
			int k, d;
		};

		inline Div MakeDiv(int d)
		{
			int l = 0;
			while ((1u << l) < (unsigned)d) l++;
			Div v;
			v.d = d;
			v.k = 31 + l;
			v.m = ((1ull << v.k) + (unsigned long long)d - 1) / (unsigned long long)d;
			return v;
		}

		__host__ __device__ __forceinline__ unsigned DivQ(unsigned n, const Div& v) { return (unsigned)(((unsigned long long)n * v.m) >> v.k); }

		// Box rows whose width is not a multiple of 32 leave the last warp of every row mostly
		// idle in the 32-wide blocks; these kernels number the points of an (x, y) plane (rows
		// of M points in y for the 2-D march) consecutively instead, so every warp but the
		// plane's last is full.  Uniform shapes only.  Launches without the march take this
		// form at every width too: a CTA then covers 256 consecutive points of one row instead
		// of 8 rows of 32 (Triton's FP64 functors over 8-11 arrays: 2.94 -> 3.14 GLUP/s); with
		// the march the 32 x 8 blocks stay faster where the rows are whole warps (GameOfLife
		// 319 against 308, the radius-4 star 146 against 142).
		template<int M, class... A>
		__global__ void Functor2DF(int x0, int y0, int y1, unsigned n, Div w, Shape s, A... args)
		{
			const unsigned idx = blockIdx.x * blockDim.x + threadIdx.x;
			if (idx >= n) return;
			const unsigned q = DivQ(idx, w);
			const int i = x0 + (int)(idx - q * (unsigned)w.d), jb = y0 + (int)q * M;
			for (int j = jb; j < jb + M && j < y1; j++) STENCIL(i, j, HolderU<A>(args, s).get()...);
		}

		template<int M, class... A>
		__global__ void Functor3DF(int x0, int y0, int z0, int z1, unsigned n, Div w, Shape s, A... args)
		{
			const unsigned idx = blockIdx.x * blockDim.x + threadIdx.x;
			if (idx >= n) return;
			const unsigned q = DivQ(idx, w);
			const int i = x0 + (int)(idx - q * (unsigned)w.d), j = y0 + (int)q;
			const int kb = z0 + (int)blockIdx.y * M;
			for (int k = kb; k < kb + M && k < z1; k++) STENCIL(i, j, k, HolderU<A>(args, s).get()...);
		}

		// The flattened launch applies: ragged rows or no march (M == 1), the plane's points
		// numbered below 2^31 and the z chunks within the grid's y limit.
		inline bool Flatten(int w, int M, long long plane, long long zchunks)
		{
			return (w % 32 != 0 || M == 1) && plane < (1ll << 31) - 256 && zchunks <= 65535;
		}

		template<int M, class... A>
		__global__ void Functor2D(int x0, int x1, int y0, int y1, A... args)
		{
			const int i = x0 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
			const int jb = y0 + (int)(blockIdx.y * blockDim.y + threadIdx.y) * M;
			if (i >= x1) return;
			for (int j = jb; j < jb + M && j < y1; j++) STENCIL(i, j, Holder<A>(args).get()...);
		}

		template<int M, class... A>
		__global__ void Functor3D(int x0, int x1, int y0, int y1, int z0, int z1, A... args)
		{
			const int i = x0 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
			const int j = y0 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
			const int kb = z0 + (int)(blockIdx.z * blockDim.z + threadIdx.z) * M;
			if (i >= x1 || j >= y1) return;
			for (int k = kb; k < kb + M && k < z1; k++) STENCIL(i, j, k, Holder<A>(args).get()...);
		}

		inline unsigned Blocks(int n, int b) { return (unsigned)((n + b - 1) / b); }

		template<class T>
		void RefreshGhosts(Grid<T>* g, bool next, cudaStream_t st = nullptr)
		{
			if (GetGhostLayer() <= 0 || !IsPeriodic() || g->GetGridType() == FLAT) return;
			Array<T>* a = next ? g->GetSubGridNextCPU() : g->GetSubGridCPU();
			const int d[3] = { a->GetDim(0), a->GetDim(1), a->GetDim(2) };
			Check(appfis_gb_ghost_periodic(next ? g->DeviceNext() : g->DeviceCurrent(), (int)sizeof(T), a->GetDimCount(), d,
				GetGhostLayer(), st ? st : GetCudaStream()), "periodic ghost refresh");
		}

		// After a sweep: refresh the updated grids' next buffers, then swap them in.
		template<class T>
		void AfterSweep(Config<T>& config)
		{
			Check(gb_launch_status(), "stencil kernel launch");
			for (size_t n = 0; n < config.updatedGrids.size(); n++) RefreshGhosts(config.updatedGrids[n], true);
			for (size_t n = 0; n < config.updatedGrids.size(); n++) config.updatedGrids[n]->Swap();
		}

		template<class T> struct DType;
		template<> struct DType<float> { static const int code = APPFIS_GB_F32; };
		template<> struct DType<double> { static const int code = APPFIS_GB_F64; };
		template<> struct DType<int> { static const int code = APPFIS_GB_I32; };
	}

	template<typename T>
	void InitializeExecution(Grid<T>& grid)
	{
		ExecutionFlag() = true;
		grid.Upload(GetCudaStream());
		if (grid.GetGridType() != FLAT)
		{
			detail::RefreshGhosts(&grid, false);  // ExchangeInitial on both buffers (Runtime.hpp:128-136)
			if (grid.GetGridType() == DUAL) detail::RefreshGhosts(&grid, true);
		}
	}

	template<typename T, typename... TArgs>
	void InitializeExecution(Grid<T>& grid, TArgs&&... args)
	{
		InitializeExecution(grid);
		InitializeExecution(args...);
	}

	template<typename T>
	void FinalizeExecution(Grid<T>& grid)
	{
		detail::FlushFast();
		ExecutionFlag() = false;
		grid.DownloadCurrent(GetCudaStream());
	}

	template<typename T, typename... TArgs>
	void FinalizeExecution(Grid<T>& grid, TArgs&&... args)
	{
		FinalizeExecution(grid);
		FinalizeExecution(args...);
	}

	namespace detail
	{
		// The functor over the box [x0, x1) x [y0, y1) on `st` (no ghost refresh, no swap).
		template<typename... TArgs>
		void Sweep2D(int x0, int x1, int y0, int y1, cudaStream_t st, TArgs... args)
		{
			if (x1 <= x0 || y1 <= y0) return;
			constexpr int M = ArrayCount<typename KArg<TArgs>::type...>::value <= MARCH_MAX_ARRAYS_2D ? MARCH : 1;
			dim3 blk(32, 8), grd(Blocks(x1 - x0, 32), Blocks(y1 - y0, 8 * M));
			Shape s;
			const bool uniform = UniformShape(s, args...);
			const long long rows = (y1 - y0 + M - 1) / M, n = (long long)(x1 - x0) * rows;
			if (uniform && Flatten(x1 - x0, M, n, 1))
				Functor2DF<M, typename KArg<TArgs>::type...><<<Blocks((int)n, 256), 256, 0, st>>>(
					x0, y0, y1, (unsigned)n, MakeDiv(x1 - x0), s, KArg<TArgs>::to(args)...);
			else if (uniform)
				Functor2DU<M, typename KArg<TArgs>::type...><<<grd, blk, 0, st>>>(x0, x1, y0, y1, s, KArg<TArgs>::to(args)...);
			else
				Functor2D<M, typename KArg<TArgs>::type...><<<grd, blk, 0, st>>>(x0, x1, y0, y1, KArg<TArgs>::to(args)...);
		}

		// The functor over the box [x0, x1) x [y0, y1) x [z0, z1) on `st`.
		template<typename... TArgs>
		void Sweep3D(int x0, int x1, int y0, int y1, int z0, int z1, cudaStream_t st, TArgs... args)
		{
			if (x1 <= x0 || y1 <= y0 || z1 <= z0) return;
			Shape s;
			const bool uniform = UniformShape(s, args...);
			const long long plane = (long long)(x1 - x0) * (y1 - y0);
			if (ArrayCount<typename KArg<TArgs>::type...>::value <= MARCH_MAX_ARRAYS)
			{
				dim3 blk(32, 8, 1), grd(Blocks(x1 - x0, 32), Blocks(y1 - y0, 8), Blocks(z1 - z0, MARCH_3D));
				if (uniform && Flatten(x1 - x0, MARCH_3D, plane, grd.z))
					Functor3DF<MARCH_3D, typename KArg<TArgs>::type...><<<dim3(Blocks((int)plane, 256), grd.z), 256, 0, st>>>(
						x0, y0, z0, z1, (unsigned)plane, MakeDiv(x1 - x0), s, KArg<TArgs>::to(args)...);
				else if (uniform)
					Functor3DU<MARCH_3D, typename KArg<TArgs>::type...><<<grd, blk, 0, st>>>(x0, x1, y0, y1, z0, z1, s,
						KArg<TArgs>::to(args)...);
				else
					Functor3D<MARCH_3D, typename KArg<TArgs>::type...><<<grd, blk, 0, st>>>(x0, x1, y0, y1, z0, z1,
						KArg<TArgs>::to(args)...);
			}
			else
			{
				dim3 blk(32, 4, 2), grd(Blocks(x1 - x0, 32), Blocks(y1 - y0, 4), Blocks(z1 - z0, 2));
				if (uniform && Flatten(x1 - x0, 1, plane, z1 - z0))
					Functor3DF<1, typename KArg<TArgs>::type...><<<dim3(Blocks((int)plane, 256), z1 - z0), 256, 0, st>>>(
						x0, y0, z0, z1, (unsigned)plane, MakeDiv(x1 - x0), s, KArg<TArgs>::to(args)...);
				else if (uniform)
					Functor3DU<1, typename KArg<TArgs>::type...><<<grd, blk, 0, st>>>(x0, x1, y0, y1, z0, z1, s, KArg<TArgs>::to(args)...);
				else
					Functor3D<1, typename KArg<TArgs>::type...><<<grd, blk, 0, st>>>(x0, x1, y0, y1, z0, z1, KArg<TArgs>::to(args)...);
			}
		}

		// The overlapped form (the reference's ExecuteOverlap*, Appfis/Runtime.hpp:372-594,
		// Runtime_CUDA.hpp:304-551: the boundary strips first, the halo exchange behind the
		// interior).  On one GPU the exchange is the periodic ghost refresh of the updated grids'
		// next buffers; it reads only the strips of width `ghost` along the box's faces, so it runs
		// on a second stream while the interior [2 ghost, dim - 2 ghost) is swept.  Applies when the
		// grids are periodic and the Config box is the whole interior with room for both parts.
		struct OverlapLane
		{
			cudaStream_t side = nullptr;
			cudaEvent_t strips = nullptr, halo = nullptr;
		};

		inline OverlapLane& Overlap()
		{
			static OverlapLane o;
			if (!o.side)
			{
				CheckCuda(cudaStreamCreateWithFlags(&o.side, cudaStreamNonBlocking), "cudaStreamCreate(overlap)");
				CheckCuda(cudaEventCreateWithFlags(&o.strips, cudaEventDisableTiming), "cudaEventCreate(overlap)");
				CheckCuda(cudaEventCreateWithFlags(&o.halo, cudaEventDisableTiming), "cudaEventCreate(overlap)");
			}
			return o;
		}

		template<class T>
		bool Overlappable(Config<T>& config, int nDim)
		{
			const int g = GetGhostLayer();
			if (!IsPeriodic() || g <= 0 || config.updatedGrids.empty()) return false;
			const int s[3] = { config.GetStartX(), config.GetStartY(), config.GetStartZ() };
			const int e[3] = { config.GetEndX(), config.GetEndY(), config.GetEndZ() };
			const int d[3] = { config.GetDimX(), config.GetDimY(), config.GetDimZ() };
			for (int a = 0; a < nDim; a++)
				if (s[a] != g || e[a] != d[a] - g || d[a] < 5 * g) return false;
			return true;
		}

		// Strips swept: refresh the updated grids' next ghosts on the side stream, behind the interior.
		template<class T>
		void OverlapHalo(Config<T>& config)
		{
			OverlapLane& o = Overlap();
			CheckCuda(cudaEventRecord(o.strips, GetCudaStream()), "overlap event");
			CheckCuda(cudaStreamWaitEvent(o.side, o.strips, 0), "overlap wait");
			for (size_t n = 0; n < config.updatedGrids.size(); n++) RefreshGhosts(config.updatedGrids[n], true, o.side);
			CheckCuda(cudaEventRecord(o.halo, o.side), "overlap event");
		}

		template<class T>
		void OverlapJoin(Config<T>& config)
		{
			Check(gb_launch_status(), "stencil kernel launch");
			CheckCuda(cudaStreamWaitEvent(GetCudaStream(), Overlap().halo, 0), "overlap wait");
			for (size_t n = 0; n < config.updatedGrids.size(); n++) config.updatedGrids[n]->Swap();
		}

		template<typename T, typename... TArgs>
		bool Routed(Config<T>& config, TArgs... args)
		{
			FastState* fs = FastFind(&config);
			if (!fs)
			{
				FlushFast();  // a functor sweep reads the grids as the deferred sweeps leave them
				return false;
			}
			FlushFast(fs);
			FastCall(*fs, config, args...);
			FastAfter(config);
			return true;
		}
	}

	// Overlapped executors (also what Execute*D runs when the Attribute asks for overlap, as the
	// reference's Execute*DGPU do: Runtime_CUDA.hpp:231-276); outside their conditions (above)
	// they are the plain sweeps.
	template<typename T, typename... TArgs>
	void ExecuteOverlap1D(Config<T>& config, TArgs... args)
	{
		if (detail::Routed(config, args...)) return;
		const int g = GetGhostLayer(), x0 = config.GetStartX(), x1 = config.GetEndX();
		if (!detail::Overlappable(config, 1))
		{
			if (x1 > x0)
				detail::Functor1D<typename detail::KArg<TArgs>::type...><<<detail::Blocks(x1 - x0, 256), 256, 0, GetCudaStream()>>>(
					x0, x1, detail::KArg<TArgs>::to(args)...);
			detail::AfterSweep(config);
			return;
		}
		cudaStream_t st = GetCudaStream();
		detail::Functor1D<typename detail::KArg<TArgs>::type...><<<detail::Blocks(g, 256), 256, 0, st>>>(x0, 2 * g,
			detail::KArg<TArgs>::to(args)...);
		detail::Functor1D<typename detail::KArg<TArgs>::type...><<<detail::Blocks(g, 256), 256, 0, st>>>(x1 - g, x1,
			detail::KArg<TArgs>::to(args)...);
		detail::OverlapHalo(config);
		detail::Functor1D<typename detail::KArg<TArgs>::type...><<<detail::Blocks(x1 - x0 - 2 * g, 256), 256, 0, st>>>(2 * g, x1 - g,
			detail::KArg<TArgs>::to(args)...);
		detail::OverlapJoin(config);
	}

	template<typename T, typename... TArgs>
	void ExecuteOverlap2D(Config<T>& config, TArgs... args)
	{
		if (detail::Routed(config, args...)) return;
		const int x0 = config.GetStartX(), x1 = config.GetEndX(), y0 = config.GetStartY(), y1 = config.GetEndY();
		cudaStream_t st = GetCudaStream();
		if (!detail::Overlappable(config, 2))
		{
			detail::Sweep2D(x0, x1, y0, y1, st, args...);
			detail::AfterSweep(config);
			return;
		}
		const int g = GetGhostLayer();
		detail::Sweep2D(x0, x1, y0, y0 + g, st, args...);          // strips along the y faces (full x)
		detail::Sweep2D(x0, x1, y1 - g, y1, st, args...);
		detail::Sweep2D(x0, x0 + g, y0 + g, y1 - g, st, args...);  // strips along the x faces
		detail::Sweep2D(x1 - g, x1, y0 + g, y1 - g, st, args...);
		detail::OverlapHalo(config);
		detail::Sweep2D(x0 + g, x1 - g, y0 + g, y1 - g, st, args...);  // interior, behind the refresh
		detail::OverlapJoin(config);
	}

	template<typename T, typename... TArgs>
	void ExecuteOverlap3D(Config<T>& config, TArgs... args)
	{
		if (detail::Routed(config, args...)) return;
		const int x0 = config.GetStartX(), x1 = config.GetEndX(), y0 = config.GetStartY(), y1 = config.GetEndY();
		const int z0 = config.GetStartZ(), z1 = config.GetEndZ();
		cudaStream_t st = GetCudaStream();
		if (!detail::Overlappable(config, 3))
		{
			detail::Sweep3D(x0, x1, y0, y1, z0, z1, st, args...);
			detail::AfterSweep(config);
			return;
		}
		const int g = GetGhostLayer();
		detail::Sweep3D(x0, x1, y0, y1, z0, z0 + g, st, args...);                  // z faces (full x, y)
		detail::Sweep3D(x0, x1, y0, y1, z1 - g, z1, st, args...);
		detail::Sweep3D(x0, x1, y0, y0 + g, z0 + g, z1 - g, st, args...);          // y faces (full x)
		detail::Sweep3D(x0, x1, y1 - g, y1, z0 + g, z1 - g, st, args...);
		detail::Sweep3D(x0, x0 + g, y0 + g, y1 - g, z0 + g, z1 - g, st, args...);  // x faces
		detail::Sweep3D(x1 - g, x1, y0 + g, y1 - g, z0 + g, z1 - g, st, args...);
		detail::OverlapHalo(config);
		detail::Sweep3D(x0 + g, x1 - g, y0 + g, y1 - g, z0 + g, z1 - g, st, args...);
		detail::OverlapJoin(config);
	}

	template<typename T, typename... TArgs>
	void Execute1D(Config<T>& config, TArgs... args)
	{
		if (IsOverlap())
		{
			ExecuteOverlap1D(config, args...);
			return;
		}
		if (detail::Routed(config, args...)) return;
		const int x0 = config.GetStartX(), x1 = config.GetEndX();
		if (x1 > x0)
			detail::Functor1D<typename detail::KArg<TArgs>::type...><<<detail::Blocks(x1 - x0, 256), 256, 0, GetCudaStream()>>>(
				x0, x1, detail::KArg<TArgs>::to(args)...);
		detail::AfterSweep(config);
	}

	template<typename T, typename... TArgs>
	void Execute2D(Config<T>& config, TArgs... args)
	{
		if (IsOverlap())
		{
			ExecuteOverlap2D(config, args...);
			return;
		}
		if (detail::Routed(config, args...)) return;
		detail::Sweep2D(config.GetStartX(), config.GetEndX(), config.GetStartY(), config.GetEndY(), GetCudaStream(), args...);
		detail::AfterSweep(config);
	}

	template<typename T, typename... TArgs>
	void Execute3D(Config<T>& config, TArgs... args)
	{
		if (IsOverlap())
		{
			ExecuteOverlap3D(config, args...);
			return;
		}
		if (detail::Routed(config, args...)) return;
		detail::Sweep3D(config.GetStartX(), config.GetEndX(), config.GetStartY(), config.GetEndY(), config.GetStartZ(),
			config.GetEndZ(), GetCudaStream(), args...);
		detail::AfterSweep(config);
	}

	namespace detail
	{
		template<typename T>
		void Reduce(Config<T>& config, T& var, REDUCTION rType, Grid<T>& grid, int nDim)
		{
			if (!grid.OnDevice())
			{
				std::cerr << "APPFIS engine: Execute*DReduce needs InitializeExecution(grid) first." << std::endl;
				std::exit(EXIT_FAILURE);
			}
			FlushFast();
			Array<T>* a = grid.GetSubGridCPU();
			const int box[6] = { config.GetStartX(), config.GetEndX(),
				nDim > 1 ? config.GetStartY() : 0, nDim > 1 ? config.GetEndY() : 1,
				nDim > 2 ? config.GetStartZ() : 0, nDim > 2 ? config.GetEndZ() : 1 };
			const int py = a->GetDimCount() > 1 ? a->GetDim(1) : 1;
			if (DType<T>::code == APPFIS_GB_I32)
			{
				// The reference accumulates an int reduction in int (Runtime.hpp:597-913), so a SUM
				// outside the int range wraps there.  The engine sums in int64; its low 32 bits are
				// that wrapped total, taken here with a defined narrowing (no double round trip).
				static long long* dres = nullptr;
				if (!dres) CheckCuda(cudaMalloc((void**)&dres, sizeof(long long)), "cudaMalloc(reduction result)");
				Check(appfis_gb_reduce(grid.DeviceCurrent(), DType<T>::code, a->GetDim(0), py, box, (int)rType, dres,
					GetCudaStream()), "reduction");
				long long v = 0;
				CheckCuda(cudaMemcpyAsync(&v, dres, sizeof v, cudaMemcpyDeviceToHost, GetCudaStream()), "reduction result copy");
				CheckCuda(cudaStreamSynchronize(GetCudaStream()), "reduction");
				var = (T)static_cast<int>(static_cast<uint32_t>(static_cast<unsigned long long>(v)));
				return;
			}
			double r = 0.0;
			Check(appfis_gb_reduce_host(grid.DeviceCurrent(), DType<T>::code, a->GetDim(0), py, box, (int)rType, &r,
				GetCudaStream()), "reduction");
			var = (T)r;
		}
	}

	template<typename T>
	void Execute1DReduce(Config<T>& config, T& var, REDUCTION rType, Grid<T>& grid) { detail::Reduce(config, var, rType, grid, 1); }

	template<typename T>
	void Execute2DReduce(Config<T>& config, T& var, REDUCTION rType, Grid<T>& grid) { detail::Reduce(config, var, rType, grid, 2); }

	template<typename T>
	void Execute3DReduce(Config<T>& config, T& var, REDUCTION rType, Grid<T>& grid) { detail::Reduce(config, var, rType, grid, 3); }

	// Checkpoint / restart of a grid's device buffers during execution (an engine extension: the
	// reference's applications checkpoint through host files after Gather, e.g. the Triton
	// restart inputs h_infile / qx_infile / qy_infile, Triton/src/config_utils.hpp:369-379).
	// Runs every deferred fast-kernel sweep first; exits with a message when the file cannot be
	// written or read (or is shorter than the grid's buffers).
	template<typename T>
	void SaveDeviceState(Grid<T>& grid, const std::string& path)
	{
		detail::FlushFast();
		if (!grid.SaveDevice(path, GetCudaStream()))
		{
			std::cerr << "APPFIS engine: cannot write the device state of a grid to " << path
				<< " (call between InitializeExecution and FinalizeExecution)" << std::endl;
			std::exit(EXIT_FAILURE);
		}
	}

	template<typename T>
	void LoadDeviceState(Grid<T>& grid, const std::string& path)
	{
		detail::FlushFast();
		if (!grid.LoadDevice(path, GetCudaStream()))
		{
			std::cerr << "APPFIS engine: cannot read the device state of a grid from " << path << std::endl;
			std::exit(EXIT_FAILURE);
		}
	}

	// Refresh the ghosts of the grid's next buffer and swap it in (Runtime.hpp:173-189).
	template<typename T>
	void HaloExchange(Grid<T>* grid)
	{
		detail::FlushFast();
		detail::RefreshGhosts(grid, true);
		grid->Swap();
	}

}

#endif

/*
 * Fast.hpp — opt-in routing of an application's Execute*D loop to the engine's hand-written
 * sweeps (no counterpart in the reference, whose every Execute*D runs the generic functor
 * kernel: Appfis/Runtime.hpp:192-222, Appfis/Runtime_CUDA.hpp:231-276).
 *
 * The engine cannot tell which functor an application wrote (Stencil overloads are free
 * functions), so the routing is explicit: one added line after the Config is set up,
 *
 *     APPFIS::UseFastKernel(config, APPFIS::FAST_LIFE);
 *
 * states that every later Execute*D(config, ...) is the named reference functor, and those calls
 * then run the matching C-ABI kernel instead:
 *
 *   FAST_LIFE          GameOfLife/src/game_appfis.hpp:121-135 (int cells, periodic, ghost 1)
 *                      -> appfis_gb_life_bits (16 generations per launch) when dimX % 32 == 0,
 *                         else appfis_gb_life_u8; bit-identical states
 *   FAST_HEAT2D        the 2-D heat functor (HeatDiffusion/src/heat_appfis.hpp:166-174 in 2-D,
 *                      float, Dirichlet ghost ring 1) -> appfis_gb_heat2d (8 sweeps per launch);
 *                      bit-identical
 *   FAST_HIMENO        Himeno/src/himeno_appfis.hpp:178-198 (float, ghost 1)
 *                      -> appfis_gb_himeno, TMA-staged (rows that are not 16-byte aligned are
 *                         run on copies with rows padded to 128 bytes); bit-identical
 *   FAST_HIMENO_MIXED  the same functor as FP16 defect correction (appfis_gb_himeno_mixed, FP32
 *                      master p refreshed every 20 sweeps); within the form's stated error
 *   FAST_STAR_R4       FDTD3d/src/fdtd3d_appfis.hpp:129-143 with radius 4 (float, ghost 4)
 *                      -> appfis_gb_star_r4 (TMA-staged when rows are 16-byte aligned); bit-identical
 *
 * The call must pass the functor's arguments in the reference's order and types (checked at
 * compile time per kernel; a mismatch exits with a message), over the Config's full interior.
 * Kernels that change layout (GameOfLife: the int grid becomes u8 or bit-packed cells) or that
 * run many sweeps per launch defer the application's sweeps and run them in one batch when the
 * grids are next observed: another Execute*D, Execute*DReduce, HaloExchange,
 * FinalizeExecution, Timer::Stop or Finalize.  The grids' buffers and their current/next roles
 * are then exactly what the functor path would have left.  Without the line nothing changes.
 */
#ifndef APPFIS_GB_FAST_HPP
#define APPFIS_GB_FAST_HPP

#include <cstdint>
#include <iostream>
#include <vector>

#include "Common.hpp"
#include "Config.hpp"
#include "Grid.hpp"

namespace APPFIS
{

	enum FAST_KERNEL { FAST_NONE = 0, FAST_LIFE, FAST_HEAT2D, FAST_HIMENO, FAST_HIMENO_MIXED, FAST_STAR_R4 };

	namespace detail
	{
		inline void FastFail(const char* what)
		{
			std::cerr << "APPFIS engine: UseFastKernel: " << what << std::endl;
			std::exit(EXIT_FAILURE);
		}

		inline void* FastAlloc(size_t bytes)
		{
			void* p = nullptr;
			CheckCuda(cudaMalloc(&p, bytes > 0 ? bytes : 16), "cudaMalloc(fast kernel buffers)");
			return p;
		}

		struct FastState
		{
			const void* key = nullptr;  // the registered Config
			FAST_KERNEL kind = FAST_NONE;
			int pending = 0;            // application sweeps not yet run
			virtual ~FastState() {}
			virtual void Flush() {}     // run the pending sweeps into the grids' own buffers
		};

		inline std::vector<FastState*>& FastStates()
		{
			static std::vector<FastState*> v;
			return v;
		}

		inline FastState* FastFind(const void* key)
		{
			for (FastState* s : FastStates())
				if (s->key == key) return s;
			return nullptr;
		}

		// Runs every deferred sweep (of all registered Configs but `except`).
		inline void FlushFast(const FastState* except = nullptr)
		{
			for (FastState* s : FastStates())
				if (s != except && s->pending) s->Flush();
		}

		inline void ReleaseFast()
		{
			FlushFast();
			for (FastState* s : FastStates()) delete s;
			FastStates().clear();
		}

		template<class T>
		bool FullInterior(const Config<T>& c, const Array<T>* a, int nDim, int g)
		{
			const int s[3] = { c.GetStartX(), c.GetStartY(), c.GetStartZ() }, e[3] = { c.GetEndX(), c.GetEndY(), c.GetEndZ() };
			if (a->GetDimCount() != nDim) return false;
			for (int d = 0; d < nDim; d++)
				if (s[d] != g || e[d] != a->GetDim(d) - g) return false;
			return true;
		}

		template<class T>
		Grid<T>* OnlyUpdatedGrid(Config<T>& c)
		{
			if (c.updatedGrids.size() != 1 || c.updatedGrids[0]->GetGridType() != DUAL)
				FastFail("the Config must update exactly one DUAL grid (GridsToUpdate)");
			return c.updatedGrids[0];
		}

		template<class U>
		U* Dev(Array<U>* a)
		{
			if (!a || !a->IsDeviceView()) FastFail("pass the grids' GetSubGrid() / GetSubGridNext() after InitializeExecution");
			return a->GetData();
		}

		// ---- GameOfLife: u8 (or bit-packed) copies of the state and of the state one generation
		// back (the reference rule keeps a cell's stale value), loaded from the int grid when a
		// run of generations starts and written back (interior + periodic ghost ring) at its end.
		struct LifeState : FastState
		{
			Grid<int>* grid = nullptr;
			int nx = 0, ny = 0, g = 1, px = 0;
			bool bits = false;
			uint8_t* u8[2] = { nullptr, nullptr };
			uint32_t* w[2] = { nullptr, nullptr };

			~LifeState()
			{
				for (int b = 0; b < 2; b++)
				{
					if (u8[b]) cudaFree(u8[b]);
					if (w[b]) cudaFree(w[b]);
				}
			}

			void Start()
			{
				const size_t n = (size_t)nx * ny;
				for (int b = 0; b < 2; b++)
				{
					if (!u8[b]) u8[b] = (uint8_t*)FastAlloc((n + 15) & ~(size_t)15);
					if (bits && !w[b]) w[b] = (uint32_t*)FastAlloc(n / 8);
				}
				cudaStream_t st = GetCudaStream();
				Check(appfis_gb_life_from_i32(grid->DeviceCurrent(), px, g, u8[0], nx, ny, st), "GameOfLife state load");
				Check(appfis_gb_life_from_i32(grid->DeviceNext(), px, g, u8[1], nx, ny, st), "GameOfLife state load");
				if (bits)
					for (int b = 0; b < 2; b++) Check(appfis_gb_life_pack(u8[b], w[b], nx, ny, st), "GameOfLife pack");
			}

			void Flush() override
			{
				if (!pending) return;
				cudaStream_t st = GetCudaStream();
				int ci = 0;
				if (bits)
				{
					Check(appfis_gb_life_bits(w[0], w[1], nx, ny, pending, APPFIS_GB_LIFE_REFERENCE, &ci, st), "GameOfLife sweeps");
					Check(appfis_gb_life_unpack(w[ci], u8[0], nx, ny, st), "GameOfLife unpack");
					Check(appfis_gb_life_unpack(w[1 - ci], u8[1], nx, ny, st), "GameOfLife unpack");
					ci = 0;
				}
				else
					Check(appfis_gb_life_u8(u8[0], u8[1], nx, ny, pending, APPFIS_GB_LIFE_REFERENCE, &ci, st), "GameOfLife sweeps");
				// newest state into the grid's current buffer, the one before it into next (the
				// roles the functor path's swaps would have left)
				Check(appfis_gb_life_to_i32(u8[ci], nx, ny, grid->DeviceCurrent(), px, g, st), "GameOfLife state store");
				Check(appfis_gb_life_to_i32(u8[1 - ci], nx, ny, grid->DeviceNext(), px, g, st), "GameOfLife state store");
				pending = 0;
			}
		};

		// ---- heat: sweeps deferred and run time-blocked on the grid's own two buffers.
		struct HeatState : FastState
		{
			Grid<float>* grid = nullptr;
			float* buf[2] = { nullptr, nullptr };  // current / next when the run of sweeps started
			float cx = 0, cy = 0;
			int nx = 0, ny = 0, px = 0;

			void Flush() override
			{
				if (!pending) return;
				int ci = 0;
				Check(appfis_gb_heat2d(buf[0], buf[1], nx, ny, px, pending, cx, cy, &ci, GetCudaStream()), "heat sweeps");
				// the grid swapped once per sweep; make its current buffer the one holding the result
				if (grid->DeviceCurrent() != buf[ci]) grid->Swap();
				pending = 0;
			}
		};

		// ---- Himeno (plain or FP16 defect correction): sweeps deferred and run in one call.  When
		// the application's rows are not 16-byte aligned (pitch not a multiple of 8 floats), the run
		// works on copies of p and the 12 coefficient fields with rows padded to 128 bytes, so the
		// TMA-staged kernels apply; p goes back into the grid's buffers at the end of the run.
		struct HimenoState : FastState
		{
			Grid<float>* grid = nullptr;
			float* buf[2] = { nullptr, nullptr };  // the grid's current / next when the run started
			const float* coef[12] = {};
			float omega = 0;
			int nx = 0, ny = 0, nz = 0, px = 0;
			// padded copies (pitch ppx): 12 coefficient fields, then the two p buffers
			float* pad = nullptr;
			size_t padBytes = 0;
			int ppx = 0;
			void* half = nullptr;
			size_t halfBytes = 0;

			~HimenoState()
			{
				if (pad) cudaFree(pad);
				if (half) cudaFree(half);
			}

			bool Padded() const { return px % 8 != 0; }
			size_t Field() const { return (size_t)(Padded() ? ppx : px) * (ny + 2) * (nz + 2); }

			void CopyRows(float* dst, int dpitch, const float* src, int spitch)
			{
				CheckCuda(cudaMemcpy2DAsync(dst, sizeof(float) * dpitch, src, sizeof(float) * spitch, sizeof(float) * (nx + 2),
					(size_t)(ny + 2) * (nz + 2), cudaMemcpyDeviceToDevice, GetCudaStream()), "Himeno padded copy");
			}

			void Start()
			{
				if (!Padded()) return;
				ppx = (nx + 2 + 31) / 32 * 32;
				const size_t need = 14 * sizeof(float) * Field();
				if (padBytes < need)
				{
					if (pad) cudaFree(pad);
					pad = (float*)FastAlloc(need);
					padBytes = need;
					CheckCuda(cudaMemsetAsync(pad, 0, need, GetCudaStream()), "Himeno padded copy");
				}
				for (int n = 0; n < 12; n++) CopyRows(pad + n * Field(), ppx, coef[n], px);
				CopyRows(pad + 12 * Field(), ppx, buf[0], px);
				CopyRows(pad + 13 * Field(), ppx, buf[1], px);
			}

			void Flush() override
			{
				if (!pending) return;
				const float* cf[12];
				float* p0 = buf[0];
				float* p1 = buf[1];
				int pitch = px;
				for (int n = 0; n < 12; n++) cf[n] = coef[n];
				if (Padded())
				{
					for (int n = 0; n < 12; n++) cf[n] = pad + n * Field();
					p0 = pad + 12 * Field();
					p1 = pad + 13 * Field();
					pitch = ppx;
				}
				int ci = 0;
				if (kind == FAST_HIMENO)
					Check(appfis_gb_himeno(cf, p0, p1, nx, ny, nz, pitch, pending, omega, nullptr, &ci, GetCudaStream()),
						"Himeno sweeps");
				else
				{
					const size_t need = 13 * sizeof(uint16_t) * Field();
					if (halfBytes < need)
					{
						if (half) cudaFree(half);
						half = FastAlloc(need);
						halfBytes = need;
					}
					Check(appfis_gb_himeno_mixed(cf, p0, p1, half, nx, ny, nz, pitch, pending, 20, omega, nullptr, &ci,
						GetCudaStream()), "Himeno defect-correction sweeps");
				}
				if (Padded())  // newest p into the buffer the run started from, the other one beside it
				{
					CopyRows(buf[0], px, ci == 0 ? p0 : p1, ppx);
					CopyRows(buf[1], px, ci == 0 ? p1 : p0, ppx);
					ci = 0;
				}
				// the grid swapped once per sweep; make its current buffer the one holding the result
				if (grid->DeviceCurrent() != buf[ci]) grid->Swap();
				pending = 0;
			}
		};

		// GameOfLife
		inline void FastCall(FastState& s, Config<int>& c, Array<int>* cur, Array<int>* next)
		{
			if (s.kind != FAST_LIFE) FastFail("these arguments are the GameOfLife functor's; the Config names another kernel");
			LifeState& L = static_cast<LifeState&>(s);
			if (!L.grid)
			{
				L.grid = OnlyUpdatedGrid(c);
				Array<int>* a = L.grid->GetSubGridCPU();
				L.g = GetGhostLayer();
				if (!IsPeriodic() || L.g != 1 || !FullInterior(c, a, 2, L.g))
					FastFail("FAST_LIFE needs a periodic 2-D grid with ghost layer 1 and the full interior as the Config box");
				L.px = a->GetDim(0);
				L.nx = a->GetDim(0) - 2;
				L.ny = a->GetDim(1) - 2;
				L.bits = L.nx % 32 == 0;
			}
			if (Dev(cur) != L.grid->DeviceCurrent() || Dev(next) != L.grid->DeviceNext())
				FastFail("FAST_LIFE: pass the updated grid's GetSubGrid(), GetSubGridNext()");
			if (!L.pending) L.Start();
			L.pending++;
		}

		// 2-D heat
		inline void FastCall(FastState& s, Config<float>& c, float cx, float cy, Array<float>* cur, Array<float>* next)
		{
			if (s.kind != FAST_HEAT2D) FastFail("these arguments are the 2-D heat functor's; the Config names another kernel");
			HeatState& H = static_cast<HeatState&>(s);
			if (!H.grid)
			{
				H.grid = OnlyUpdatedGrid(c);
				Array<float>* a = H.grid->GetSubGridCPU();
				if (IsPeriodic() || GetGhostLayer() != 1 || !FullInterior(c, a, 2, 1))
					FastFail("FAST_HEAT2D needs a non-periodic 2-D grid with ghost layer 1 and the full interior as the Config box");
				H.px = a->GetDim(0);
				H.nx = a->GetDim(0) - 2;
				H.ny = a->GetDim(1) - 2;
			}
			if (Dev(cur) != H.grid->DeviceCurrent() || Dev(next) != H.grid->DeviceNext())
				FastFail("FAST_HEAT2D: pass the updated grid's GetSubGrid(), GetSubGridNext()");
			if (H.pending && (cx != H.cx || cy != H.cy)) H.Flush();  // one batch per set of coefficients
			if (!H.pending)
			{
				H.buf[0] = H.grid->DeviceCurrent();
				H.buf[1] = H.grid->DeviceNext();
				H.cx = cx;
				H.cy = cy;
			}
			H.pending++;
		}

		// Himeno (plain or FP16 defect correction; deferred)
		inline void FastCall(FastState& s, Config<float>& c, float omega, Array<float>* a0, Array<float>* a1, Array<float>* a2,
			Array<float>* a3, Array<float>* b0, Array<float>* b1, Array<float>* b2, Array<float>* c0, Array<float>* c1,
			Array<float>* c2, Array<float>* bnd, Array<float>* wrk1, Array<float>* p, Array<float>* wrk2)
		{
			if (s.kind != FAST_HIMENO && s.kind != FAST_HIMENO_MIXED)
				FastFail("these arguments are the Himeno functor's; the Config names another kernel");
			Grid<float>* grid = OnlyUpdatedGrid(c);
			Array<float>* shape = grid->GetSubGridCPU();
			if (IsPeriodic() || GetGhostLayer() != 1 || !FullInterior(c, shape, 3, 1))
				FastFail("FAST_HIMENO needs a non-periodic 3-D grid with ghost layer 1 and the full interior as the Config box");
			Array<float>* cf[12] = { a0, a1, a2, a3, b0, b1, b2, c0, c1, c2, bnd, wrk1 };
			const float* coef[12];
			for (int n = 0; n < 12; n++)
			{
				coef[n] = Dev(cf[n]);
				if (cf[n]->GetSize() != shape->GetSize()) FastFail("FAST_HIMENO: coefficient grids must have the p grid's shape");
			}
			float* pd = Dev(p);
			float* wd = Dev(wrk2);
			if (pd != grid->DeviceCurrent() || wd != grid->DeviceNext())
				FastFail("FAST_HIMENO: pass the updated grid's GetSubGrid(), GetSubGridNext() as p, wrk2");
			HimenoState& H = static_cast<HimenoState&>(s);
			bool same = H.pending && omega == H.omega;
			for (int n = 0; n < 12 && same; n++) same = coef[n] == H.coef[n];
			if (H.pending && !same) H.Flush();  // one run per set of coefficient fields and omega
			if (!H.pending)
			{
				H.grid = grid;
				H.buf[0] = pd;
				H.buf[1] = wd;
				for (int n = 0; n < 12; n++) H.coef[n] = coef[n];
				H.omega = omega;
				H.px = shape->GetDim(0);
				H.nx = H.px - 2;
				H.ny = shape->GetDim(1) - 2;
				H.nz = shape->GetDim(2) - 2;
				H.Start();
			}
			H.pending++;
		}

		// FDTD3d radius-4 star (reference form): one launch per call on the grid's buffers
		inline void FastCall(FastState& s, Config<float>& c, float coeff, int radius, Array<float>* cur, Array<float>* next)
		{
			if (s.kind != FAST_STAR_R4) FastFail("these arguments are the FDTD3d functor's; the Config names another kernel");
			Grid<float>* grid = OnlyUpdatedGrid(c);
			Array<float>* a = grid->GetSubGridCPU();
			if (radius != 4 || GetGhostLayer() != 4 || IsPeriodic() || !FullInterior(c, a, 3, 4))
				FastFail("FAST_STAR_R4 needs radius 4, ghost layer 4, a non-periodic 3-D grid and the full interior as the Config box");
			float* cd = Dev(cur);
			float* nd = Dev(next);
			if (cd != grid->DeviceCurrent() || nd != grid->DeviceNext())
				FastFail("FAST_STAR_R4: pass the updated grid's GetSubGrid(), GetSubGridNext()");
			const int px = a->GetDim(0);
			int ci = 1;
			Check(appfis_gb_star_r4(cd, nd, APPFIS_GB_F32, px - 8, a->GetDim(1) - 8, a->GetDim(2) - 8, px, 1, 0, coeff, nullptr,
				APPFIS_GB_STAR_AUTO, 0, &ci, GetCudaStream()), "radius-4 star sweep");
			if (ci != 1) FastFail("FAST_STAR_R4: the sweep's result is not in the next buffer");
		}

		// Any other argument list: not one of the kernels above.
		template<class T, class... A>
		void FastCall(FastState&, Config<T>&, A...)
		{
			FastFail("the arguments of this Execute*D call match none of the fast kernels (check the functor's argument types)");
		}

		// After a routed call: the same grid roles as after a functor sweep (the fast kernels keep
		// the ghost rings themselves: constant Dirichlet rings, or GameOfLife's wrap).
		template<class T>
		void FastAfter(Config<T>& c)
		{
			for (size_t n = 0; n < c.updatedGrids.size(); n++) c.updatedGrids[n]->Swap();
		}
	}

	// Routes every later Execute*D(config, ...) to the named hand-written kernel (see above);
	// FAST_NONE goes back to the functor path.
	template<typename T>
	void UseFastKernel(Config<T>& config, FAST_KERNEL kind)
	{
		detail::FlushFast();
		std::vector<detail::FastState*>& v = detail::FastStates();
		for (size_t n = 0; n < v.size(); n++)
			if (v[n]->key == &config)
			{
				delete v[n];
				v.erase(v.begin() + (long)n);
				break;
			}
		if (kind == FAST_NONE) return;
		detail::FastState* s = nullptr;
		switch (kind)
		{
		case FAST_LIFE: s = new detail::LifeState(); break;
		case FAST_HEAT2D: s = new detail::HeatState(); break;
		case FAST_HIMENO:
		case FAST_HIMENO_MIXED: s = new detail::HimenoState(); break;
		case FAST_STAR_R4: s = new detail::FastState(); break;
		default: detail::FastFail("unknown kernel");
		}
		s->key = &config;
		s->kind = kind;
		v.push_back(s);
		Context& ctx = Context::Get();
		ctx.flushFast = []() { detail::FlushFast(); };
		ctx.releaseFast = []() { detail::ReleaseFast(); };
	}

}

#endif

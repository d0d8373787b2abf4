// Drop-in test program: functors written the way APPFIS applications write them (free
// APPFIS::Stencil overloads on Array pointers, driven by Grid / Config / Execute*D /
// Execute*DReduce / HaloExchange), built against the engine's drop-in headers
// (appfis_gb300/Appfis) and run on the GPU.  tests/test_dropin_gpu.py compares its outputs
// with the oracle.  The functors restate the reference applications' (file:line per functor);
// the flood-model fluxes reuse the engine's own device face solver (flood_core.cuh).
//
// usage: dropin_runner gol    NX NY GENS in.u8 out.u8
//        dropin_runner heat2d NX NY ITERS R TOP in.f32 out.f32
//        dropin_runner himeno NX NY NZ ITERS OMEGA coef.f32 p.f32 out.f32
//        dropin_runner fdtd   NX NY NZ ITERS COEFF in.f32 out.f32
//        dropin_runner triton NX NY DX CN HEXTRA MANN T_END PRINT TSTEP MAXSTEPS dem.f64 h.f64 out.f64 dt.f64
//        dropin_runner ireduce NX NY in.i32           (Execute2DReduce SUM / MAX / MIN of an int grid)
//        dropin_runner star_periodic NX NY NZ ITERS in.f32 plain.f32 overlap.f32
//                      the radius-4 star on a PERIODIC grid, once with Execute3D and once with
//                      ExecuteOverlap3D (boundary slabs, then the ghost refresh behind the interior)
//        dropin_runner ckpt NX NY G1 G2 in.u8 a.u8 b.u8 DIR [fast]
//                      GameOfLife: G1 generations, SaveDeviceState, G2 more -> a; a second grid
//                      restored with LoadDeviceState, G2 generations -> b (a == b == G1 + G2
//                      generations); Array::Save/LoadBinaryFile round trip of the gathered grid
// A trailing word routes the Execute loop to a hand-written kernel (APPFIS::UseFastKernel):
//        heat2d ... fast | himeno ... fast | himeno ... mixed | fdtd ... fast | gol ... fast
#include <cfloat>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../appfis_gb300/Appfis/Appfis.hpp"
#include "../../appfis_gb300/csrc/flood_core.cuh"

namespace APPFIS
{
	// GameOfLife/src/game_appfis.hpp:121-135
	PARALLEL void STENCIL(const int i, const int j, Array<int>* cur, Array<int>* next)
	{
		int count = cur->Get(i - 1, j - 1) + cur->Get(i, j - 1) + cur->Get(i + 1, j - 1) + cur->Get(i - 1, j) + cur->Get(i + 1, j)
			+ cur->Get(i - 1, j + 1) + cur->Get(i, j + 1) + cur->Get(i + 1, j + 1);
		if (cur->Get(i, j) == 1)
		{
			if (count < 2 || count > 4) next->Set(i, j, 0);
		}
		else if (count == 3)
			next->Set(i, j, 1);
	}

	// HeatDiffusion/src/heat_appfis.hpp:166-174 in 2-D FP32; explicit rounding keeps the
	// CPU operation order (no FMA contraction)
	PARALLEL void STENCIL(const int i, const int j, float cx, float cy, Array<float>* cur, Array<float>* next)
	{
		const float c = cur->Get(i, j), two_c = __fmul_rn(2.0f, c);
		const float x = __fmul_rn(cx, __fsub_rn(__fadd_rn(cur->Get(i - 1, j), cur->Get(i + 1, j)), two_c));
		const float y = __fmul_rn(cy, __fsub_rn(__fadd_rn(cur->Get(i, j - 1), cur->Get(i, j + 1)), two_c));
		next->Set(i, j, __fadd_rn(__fadd_rn(c, x), y));
	}

	// Himeno/src/himeno_appfis.hpp:178-198 (same order, explicit rounding)
	PARALLEL void STENCIL(const int i, const int j, const int k, float omega, Array<float>* a0, Array<float>* a1, Array<float>* a2,
		Array<float>* a3, Array<float>* b0, Array<float>* b1, Array<float>* b2, Array<float>* c0, Array<float>* c1,
		Array<float>* c2, Array<float>* bnd, Array<float>* wrk1, Array<float>* p, Array<float>* wrk2)
	{
#define P(a, b, c) p->Get(i + (a), j + (b), k + (c))
		float s0 = __fmul_rn(a0->Get(i, j, k), P(1, 0, 0));
		s0 = __fadd_rn(s0, __fmul_rn(a1->Get(i, j, k), P(0, 1, 0)));
		s0 = __fadd_rn(s0, __fmul_rn(a2->Get(i, j, k), P(0, 0, 1)));
		s0 = __fadd_rn(s0, __fmul_rn(b0->Get(i, j, k), __fadd_rn(__fsub_rn(__fsub_rn(P(1, 1, 0), P(1, -1, 0)), P(-1, 1, 0)), P(-1, -1, 0))));
		s0 = __fadd_rn(s0, __fmul_rn(b1->Get(i, j, k), __fadd_rn(__fsub_rn(__fsub_rn(P(0, 1, 1), P(0, -1, 1)), P(0, 1, -1)), P(0, -1, -1))));
		s0 = __fadd_rn(s0, __fmul_rn(b2->Get(i, j, k), __fadd_rn(__fsub_rn(__fsub_rn(P(1, 0, 1), P(-1, 0, 1)), P(1, 0, -1)), P(-1, 0, -1))));
		s0 = __fadd_rn(s0, __fmul_rn(c0->Get(i, j, k), P(-1, 0, 0)));
		s0 = __fadd_rn(s0, __fmul_rn(c1->Get(i, j, k), P(0, -1, 0)));
		s0 = __fadd_rn(s0, __fmul_rn(c2->Get(i, j, k), P(0, 0, -1)));
		s0 = __fadd_rn(s0, wrk1->Get(i, j, k));
		const float ss = __fmul_rn(__fsub_rn(__fmul_rn(s0, a3->Get(i, j, k)), P(0, 0, 0)), bnd->Get(i, j, k));
		wrk2->Set(i, j, k, __fadd_rn(P(0, 0, 0), __fmul_rn(omega, ss)));
#undef P
	}

	// FDTD3d/src/fdtd3d_appfis.hpp:129-143
	PARALLEL void STENCIL(const int i, const int j, const int k, float coeff, int radius, Array<float>* cur, Array<float>* next)
	{
		float val = cur->Get(i, j, k);
		for (int a = 1; a <= radius; a++)
			val += (cur->Get(i - a, j, k) + cur->Get(i + a, j, k)) + (cur->Get(i, j - a, k) + cur->Get(i, j + a, k))
				+ (cur->Get(i, j, k - a) + cur->Get(i, j, k + a));
		val *= coeff;
		next->Set(i, j, k, val);
	}

	// ---- flood model (Triton/src/triton_appfis.hpp:567-1112), FP64
	// CFL dt per cell (:567-586)
	PARALLEL void STENCIL(const int i, const int j, double dx, double cn, double hextra, Array<double>* qx, Array<double>* qy,
		Array<double>* h, Array<double>* out)
	{
		out->Set(i, j, DBL_MAX);
		const double hij = h->Get(i, j);
		if (hij > hextra)
		{
			const double dtx = dx / (fabs(qx->Get(i, j) / hij) + sqrt(9.81 * hij));
			const double dty = dx / (fabs(qy->Get(i, j) / hij) + sqrt(9.81 * hij));
			out->Set(i, j, dtx < dty ? cn * dtx : cn * dty);
		}
	}

	// sqrt(h) and RHS reset over the whole field (:589-605)
	PARALLEL void STENCIL(const int i, const int j, Array<double>* h, Array<double>* sq, Array<double>* r0, Array<double>* r1,
		Array<double>* r2, Array<double>* r3, Array<double>* r4, Array<double>* r5)
	{
		const double hij = h->Get(i, j);
		sq->Set(i, j, hij > 0.0 ? sqrt(hij) : 0.0);
		r0->Set(i, j, 0.0);
		r1->Set(i, j, 0.0);
		r2->Set(i, j, 0.0);
		r3->Set(i, j, 0.0);
		r4->Set(i, j, 0.0);
		r5->Set(i, j, 0.0);
	}

	__device__ inline flood::Cell<double> CellAt(Array<double>* h, Array<double>* qx, Array<double>* qy, Array<double>* z,
		Array<double>* sq, int i, int j)
	{
		flood::Cell<double> c;
		c.h = h->Get(i, j);
		c.qx = qx->Get(i, j);
		c.qy = qy->Get(i, j);
		c.z = z->Get(i, j);
		c.sq = sq->Get(i, j);
		return c;
	}

	// X faces ii|ii+1, RHS set (:608-824)
	PARALLEL void STENCIL(const int ii, const int jj, double dx, double dt, double hextra, Array<double>* h, Array<double>* qx,
		Array<double>* qy, Array<double>* z, Array<double>* sq, Array<double>* rh0, Array<double>* rh1, Array<double>* rx0,
		Array<double>* rx1, Array<double>* ry0, Array<double>* ry1)
	{
		double r1[3], r2[3];
		if (!flood::face<double>(CellAt(h, qx, qy, z, sq, ii, jj), CellAt(h, qx, qy, z, sq, ii + 1, jj), 1.0, 0.0, dx, dt, hextra, r1, r2)) return;
		rh0->Set(ii, jj, r1[0]);
		rx0->Set(ii, jj, r1[1]);
		ry0->Set(ii, jj, r1[2]);
		rh1->Set(ii + 1, jj, r2[0]);
		rx1->Set(ii + 1, jj, r2[1]);
		ry1->Set(ii + 1, jj, r2[2]);
	}

	// Y faces jj|jj-1, RHS accumulated (:827-1043); `dummy` selects this overload, as in the reference
	PARALLEL void STENCIL(const int ii, const int jj, double dx, double dt, double hextra, int dummy, Array<double>* h,
		Array<double>* qx, Array<double>* qy, Array<double>* z, Array<double>* sq, Array<double>* rh0, Array<double>* rh1,
		Array<double>* rx0, Array<double>* rx1, Array<double>* ry0, Array<double>* ry1)
	{
		double r1[3], r2[3];
		if (!flood::face<double>(CellAt(h, qx, qy, z, sq, ii, jj), CellAt(h, qx, qy, z, sq, ii, jj - 1), 0.0, 1.0, dx, dt, hextra, r1, r2)) return;
		rh0->Set(ii, jj, rh0->Get(ii, jj) + r1[0]);
		rx0->Set(ii, jj, rx0->Get(ii, jj) + r1[1]);
		ry0->Set(ii, jj, ry0->Get(ii, jj) + r1[2]);
		rh1->Set(ii, jj - 1, rh1->Get(ii, jj - 1) + r2[0]);
		rx1->Set(ii, jj - 1, rx1->Get(ii, jj - 1) + r2[1]);
		ry1->Set(ii, jj - 1, ry1->Get(ii, jj - 1) + r2[2]);
	}

	// update + Manning friction (:1046-1092)
	PARALLEL void STENCIL(const int i, const int j, double dt, double hextra, Array<double>* h, Array<double>* qx, Array<double>* qy,
		Array<double>* z, Array<double>* n2, Array<double>* rh0, Array<double>* rh1, Array<double>* rx0, Array<double>* rx1,
		Array<double>* ry0, Array<double>* ry1)
	{
		const double r0[3] = { rh0->Get(i, j), rx0->Get(i, j), ry0->Get(i, j) };
		const double r1[3] = { rh1->Get(i, j), rx1->Get(i, j), ry1->Get(i, j) };
		double ho, qxo, qyo;
		flood::update<double>(h->Get(i, j), qx->Get(i, j), qy->Get(i, j), n2->Get(i, j), r0, r1, dt, hextra, ho, qxo, qyo);
		h->Set(i, j, ho);
		qx->Set(i, j, qxo);
		qy->Set(i, j, qyo);
	}

	// wet/dry momentum fix (:1095-1112)
	PARALLEL void STENCIL(const int i, const int j, double dt, double hextra, Array<double>* h, Array<double>* qx, Array<double>* qy,
		Array<double>* z)
	{
		const double hij = h->Get(i, j), lvl = hij + z->Get(i, j);
		if (hij > hextra)
		{
			if ((lvl < z->Get(i + 1, j) && h->Get(i + 1, j) < 1e-12) || (lvl < z->Get(i - 1, j) && h->Get(i - 1, j) < 1e-12)) qx->Set(i, j, 0.0);
			if ((lvl < z->Get(i, j - 1) && h->Get(i, j - 1) < 1e-12) || (lvl < z->Get(i, j + 1) && h->Get(i, j + 1) < 1e-12)) qy->Set(i, j, 0.0);
		}
	}
}

static std::vector<char> ReadFile(const char* path, size_t bytes)
{
	std::vector<char> b(bytes);
	FILE* f = std::fopen(path, "rb");
	if (!f || std::fread(b.data(), 1, bytes, f) != bytes)
	{
		std::fprintf(stderr, "cannot read %zu bytes from %s\n", bytes, path);
		std::exit(2);
	}
	std::fclose(f);
	return b;
}

static void WriteFile(const char* path, const void* p, size_t bytes)
{
	FILE* f = std::fopen(path, "wb");
	if (!f)
	{
		std::fprintf(stderr, "cannot write %s\n", path);
		std::exit(2);
	}
	std::fwrite(p, 1, bytes, f);
	std::fclose(f);
}

// The trailing routing word at argv[at], if any.
static APPFIS::FAST_KERNEL Routing(int argc, char** argv, int at, APPFIS::FAST_KERNEL fast)
{
	if (argc <= at) return APPFIS::FAST_NONE;
	const std::string w(argv[at]);
	if (w == "fast") return fast;
	if (w == "mixed") return APPFIS::FAST_HIMENO_MIXED;
	return APPFIS::FAST_NONE;
}

static int RunGol(int argc, char** argv)
{
	const int nx = std::atoi(argv[2]), ny = std::atoi(argv[3]), gens = std::atoi(argv[4]);
	std::vector<char> in = ReadFile(argv[5], (size_t)nx * ny);
	APPFIS::Attribute attr;
	attr.ghostLayer = 1;
	attr.periodic = true;
	APPFIS::Initialize(argc, argv, APPFIS::DIM_2D, APPFIS::DIM_2D, attr);
	APPFIS::Grid<int> g(APPFIS::DIM_2D, nx, ny, APPFIS::DUAL);
	g.AllocateFullGrid();
	for (int j = 0; j < ny; j++)
		for (int i = 0; i < nx; i++) g.GetFullGrid()->Set(i, j, (int)(unsigned char)in[(size_t)j * nx + i]);
	APPFIS::Scatter(g.GetFullGrid(), g.GetSubGrid());
	APPFIS::Config<int> config(g);
	config.GridsToUpdate(g);
	APPFIS::UseFastKernel(config, Routing(argc, argv, 7, APPFIS::FAST_LIFE));
	APPFIS::InitializeExecution(g);
	APPFIS::Timer timer;
	timer.Start("COMPUTE");
	for (int t = 0; t < gens; t++)  // the overlapped executor is the same sweep: alternate the two
	{
		if (t & 1)
			APPFIS::ExecuteOverlap2D(config, g.GetSubGrid(), g.GetSubGridNext());
		else
			APPFIS::Execute2D(config, g.GetSubGrid(), g.GetSubGridNext());
	}
	timer.Stop("COMPUTE");
	int live = 0;
	APPFIS::Execute2DReduce(config, live, APPFIS::SUM, g);
	APPFIS::FinalizeExecution(g);
	APPFIS::Gather(g.GetFullGrid(), g.GetSubGrid());
	std::vector<unsigned char> out((size_t)nx * ny);
	for (int j = 0; j < ny; j++)
		for (int i = 0; i < nx; i++) out[(size_t)j * nx + i] = (unsigned char)g.GetFullGrid()->Get(i, j);
	WriteFile(argv[6], out.data(), out.size());
	std::printf("{\"live\": %d, \"seconds\": %.9f}\n", live, timer.GetCustomTime("COMPUTE"));
	APPFIS::Finalize();
	return 0;
}

static int RunHeat2d(int argc, char** argv)
{
	const int nx = std::atoi(argv[2]), ny = std::atoi(argv[3]), iters = std::atoi(argv[4]);
	const float r = (float)std::atof(argv[5]), top = (float)std::atof(argv[6]);
	std::vector<char> in = ReadFile(argv[7], sizeof(float) * (size_t)nx * ny);
	const float* src = reinterpret_cast<const float*>(in.data());
	APPFIS::Attribute attr;
	APPFIS::Initialize(argc, argv, APPFIS::DIM_2D, APPFIS::DIM_2D, attr);
	APPFIS::Grid<float> g(APPFIS::DIM_2D, nx, ny, APPFIS::DUAL);
	g.AllocateFullGrid();
	for (int j = 0; j < ny; j++)
		for (int i = 0; i < nx; i++) g.GetFullGrid()->Set(i, j, src[(size_t)j * nx + i]);
	APPFIS::Scatter(g.GetFullGrid(), g.GetSubGrid());
	g.SetBoundary(0.0f);
	g.SetBoundary(APPFIS::UP, top);
	APPFIS::Config<float> config(g);
	config.GridsToUpdate(g);
	APPFIS::UseFastKernel(config, Routing(argc, argv, 9, APPFIS::FAST_HEAT2D));
	APPFIS::InitializeExecution(g);
	for (int t = 0; t < iters; t++) APPFIS::Execute2D(config, r, r, g.GetSubGrid(), g.GetSubGridNext());
	float mx = 0, mn = 0, sm = 0;
	APPFIS::Execute2DReduce(config, mx, APPFIS::MAX, g);
	APPFIS::Execute2DReduce(config, mn, APPFIS::MIN, g);
	APPFIS::Execute2DReduce(config, sm, APPFIS::SUM, g);
	APPFIS::FinalizeExecution(g);
	APPFIS::Array<float>* sub = g.GetSubGrid();
	WriteFile(argv[8], sub->GetData(), sizeof(float) * (size_t)sub->GetSize());
	std::printf("{\"max\": %.9g, \"min\": %.9g, \"sum\": %.9g}\n", mx, mn, sm);
	APPFIS::Finalize();
	return 0;
}

static int RunHimeno(int argc, char** argv)
{
	const int nx = std::atoi(argv[2]), ny = std::atoi(argv[3]), nz = std::atoi(argv[4]), iters = std::atoi(argv[5]);
	const float omega = (float)std::atof(argv[6]);
	const size_t padded = (size_t)(nx + 2) * (ny + 2) * (nz + 2);
	std::vector<char> coef = ReadFile(argv[7], 12 * padded * sizeof(float));
	std::vector<char> pin = ReadFile(argv[8], (size_t)nx * ny * nz * sizeof(float));
	APPFIS::Attribute attr;
	APPFIS::Initialize(argc, argv, APPFIS::DIM_3D, APPFIS::DIM_3D, attr);
	APPFIS::Grid<float> gp(APPFIS::DIM_3D, nx, ny, nz, APPFIS::DUAL);
	std::vector<APPFIS::Grid<float>*> gc;
	for (int c = 0; c < 12; c++) gc.push_back(new APPFIS::Grid<float>(APPFIS::DIM_3D, nx, ny, nz, APPFIS::SINGLE));
	gp.AllocateFullGrid();
	std::memcpy(gp.GetFullGrid()->GetData(), pin.data(), pin.size());
	APPFIS::Scatter(gp.GetFullGrid(), gp.GetSubGrid());
	for (int c = 0; c < 12; c++) gc[c]->GetSubGrid()->SetData(reinterpret_cast<float*>(coef.data()) + c * padded);
	APPFIS::Config<float> config(gp);
	config.GridsToUpdate(gp);
	APPFIS::UseFastKernel(config, Routing(argc, argv, 10, APPFIS::FAST_HIMENO));
	APPFIS::InitializeExecution(gp, *gc[0], *gc[1], *gc[2], *gc[3], *gc[4], *gc[5], *gc[6], *gc[7], *gc[8], *gc[9], *gc[10], *gc[11]);
	for (int t = 0; t < iters; t++)
		APPFIS::Execute3D(config, omega, gc[0]->GetSubGrid(), gc[1]->GetSubGrid(), gc[2]->GetSubGrid(), gc[3]->GetSubGrid(),
			gc[4]->GetSubGrid(), gc[5]->GetSubGrid(), gc[6]->GetSubGrid(), gc[7]->GetSubGrid(), gc[8]->GetSubGrid(),
			gc[9]->GetSubGrid(), gc[10]->GetSubGrid(), gc[11]->GetSubGrid(), gp.GetSubGrid(), gp.GetSubGridNext());
	float sum = 0;
	APPFIS::Execute3DReduce(config, sum, APPFIS::SUM, gp);
	APPFIS::FinalizeExecution(gp);
	WriteFile(argv[9], gp.GetSubGrid()->GetData(), sizeof(float) * padded);
	std::printf("{\"sum\": %.9g}\n", sum);
	for (int c = 0; c < 12; c++) delete gc[c];
	APPFIS::Finalize();
	return 0;
}

static int RunFdtd(int argc, char** argv)
{
	const int nx = std::atoi(argv[2]), ny = std::atoi(argv[3]), nz = std::atoi(argv[4]), iters = std::atoi(argv[5]);
	const float coeff = (float)std::atof(argv[6]);
	const int radius = 4;
	std::vector<char> in = ReadFile(argv[7], (size_t)nx * ny * nz * sizeof(float));
	APPFIS::Attribute attr;
	attr.ghostLayer = radius;
	APPFIS::Initialize(argc, argv, APPFIS::DIM_3D, APPFIS::DIM_3D, attr);
	APPFIS::Grid<float> g(APPFIS::DIM_3D, nx, ny, nz, APPFIS::DUAL);
	g.AllocateFullGrid();
	std::memcpy(g.GetFullGrid()->GetData(), in.data(), in.size());
	APPFIS::Scatter(g.GetFullGrid(), g.GetSubGrid());
	APPFIS::Config<float> config(g);
	config.GridsToUpdate(g);
	APPFIS::UseFastKernel(config, Routing(argc, argv, 9, APPFIS::FAST_STAR_R4));
	APPFIS::InitializeExecution(g);
	for (int t = 0; t < iters; t++) APPFIS::Execute3D(config, coeff, radius, g.GetSubGrid(), g.GetSubGridNext());
	APPFIS::FinalizeExecution(g);
	APPFIS::Array<float>* sub = g.GetSubGrid();
	WriteFile(argv[8], sub->GetData(), sizeof(float) * (size_t)sub->GetSize());
	std::printf("{\"ok\": 1}\n");
	APPFIS::Finalize();
	return 0;
}

// The reference time loop (Triton/src/triton_appfis.hpp:316-386) without sources.
static int RunTriton(int argc, char** argv)
{
	const int nx = std::atoi(argv[2]), ny = std::atoi(argv[3]);
	const double cell = std::atof(argv[4]), courant = std::atof(argv[5]), hextra = std::atof(argv[6]), mann = std::atof(argv[7]);
	const double t_end = std::atof(argv[8]), print_interval = std::atof(argv[9]), time_step = std::atof(argv[10]);
	const int max_steps = std::atoi(argv[11]);
	const size_t n = (size_t)nx * ny;
	std::vector<char> demb = ReadFile(argv[12], n * sizeof(double)), hb = ReadFile(argv[13], n * sizeof(double));
	APPFIS::Attribute attr;
	APPFIS::Initialize(argc, argv, APPFIS::DIM_2D, APPFIS::DIM_2D, attr);
	typedef APPFIS::Grid<double> GD;
	GD dem(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE), nin(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE);
	GD hin(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE), uin(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE), vin(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE);
	GD sqrth(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE);
	GD rh0(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE), rh1(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE), rx0(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE);
	GD rx1(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE), ry0(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE), ry1(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE);
	GD dtv(APPFIS::DIM_2D, nx, ny, APPFIS::DUAL);
	dem.AllocateFullGrid();
	nin.AllocateFullGrid();
	hin.AllocateFullGrid();
	std::memcpy(dem.GetFullGrid()->GetData(), demb.data(), demb.size());
	std::memcpy(hin.GetFullGrid()->GetData(), hb.data(), hb.size());
	nin.GetFullGrid()->FillData(mann);
	nin.GetFullGrid()->Square();
	APPFIS::Scatter(dem.GetFullGrid(), dem.GetSubGrid());
	dem.SetBoundary(1e6);
	APPFIS::Scatter(nin.GetFullGrid(), nin.GetSubGrid());
	nin.SetBoundaryCopy();
	APPFIS::Scatter(hin.GetFullGrid(), hin.GetSubGrid());

	APPFIS::Config<double> config(dem), configF(dem, 0, 0, 0, 0), configX(dem, 0, 1, 1, 1), configY(dem, 1, 1, 1, 0), configQ(dem);
	configQ.GridsToUpdate(uin, vin);
	APPFIS::InitializeExecution(dem, nin, hin, uin, vin, sqrth, rh0, rh1, rx0, rx1, ry0, ry1, dtv);

	double simtime = 0.0, dt = time_step;
	int steps = 0, print_id = 0;
	std::vector<double> dts;
	while (simtime < t_end && (max_steps <= 0 || steps < max_steps))
	{
		steps++;
		APPFIS::Execute2D(config, cell, courant, hextra, uin.GetSubGrid(), vin.GetSubGrid(), hin.GetSubGrid(), dtv.GetSubGrid());
		APPFIS::Execute2DReduce(config, dt, APPFIS::MIN, dtv);
		if (dt >= DBL_MAX - 1.0) dt = time_step;
		if (simtime + dt > print_interval * (print_id + 1)) dt = print_interval * (print_id + 1) - simtime;
		APPFIS::Execute2D(configF, hin.GetSubGrid(), sqrth.GetSubGrid(), rh0.GetSubGrid(), rh1.GetSubGrid(), rx0.GetSubGrid(),
			rx1.GetSubGrid(), ry0.GetSubGrid(), ry1.GetSubGrid());
		APPFIS::Execute2D(configX, cell, dt, hextra, hin.GetSubGrid(), uin.GetSubGrid(), vin.GetSubGrid(), dem.GetSubGrid(),
			sqrth.GetSubGrid(), rh0.GetSubGrid(), rh1.GetSubGrid(), rx0.GetSubGrid(), rx1.GetSubGrid(), ry0.GetSubGrid(), ry1.GetSubGrid());
		APPFIS::Execute2D(configY, cell, dt, hextra, 0, hin.GetSubGrid(), uin.GetSubGrid(), vin.GetSubGrid(), dem.GetSubGrid(),
			sqrth.GetSubGrid(), rh0.GetSubGrid(), rh1.GetSubGrid(), rx0.GetSubGrid(), rx1.GetSubGrid(), ry0.GetSubGrid(), ry1.GetSubGrid());
		APPFIS::Execute2D(config, dt, hextra, hin.GetSubGrid(), uin.GetSubGrid(), vin.GetSubGrid(), dem.GetSubGrid(), nin.GetSubGrid(),
			rh0.GetSubGrid(), rh1.GetSubGrid(), rx0.GetSubGrid(), rx1.GetSubGrid(), ry0.GetSubGrid(), ry1.GetSubGrid());
		APPFIS::HaloExchange(&hin);
		APPFIS::Execute2D(configQ, dt, hextra, hin.GetSubGrid(), uin.GetSubGrid(), vin.GetSubGrid(), dem.GetSubGrid());
		simtime += dt;
		dts.push_back(dt);
		if (simtime >= print_interval * (print_id + 1)) print_id++;
	}
	APPFIS::FinalizeExecution(hin, uin, vin);
	std::vector<double> out(3 * n);
	for (int j = 0; j < ny; j++)
		for (int i = 0; i < nx; i++)
		{
			const size_t c = (size_t)j * nx + i;
			out[c] = hin.GetSubGrid()->Get(i + 1, j + 1);
			out[n + c] = uin.GetSubGrid()->Get(i + 1, j + 1);
			out[2 * n + c] = vin.GetSubGrid()->Get(i + 1, j + 1);
		}
	WriteFile(argv[14], out.data(), out.size() * sizeof(double));
	WriteFile(argv[15], dts.data(), dts.size() * sizeof(double));
	std::printf("{\"steps\": %d, \"simtime\": %.17g}\n", steps, simtime);
	APPFIS::Finalize();
	return 0;
}

// int reductions: the reference accumulates in int, so a SUM outside the int range wraps
static int RunIntReduce(int argc, char** argv)
{
	const int nx = std::atoi(argv[2]), ny = std::atoi(argv[3]);
	std::vector<char> in = ReadFile(argv[4], sizeof(int) * (size_t)nx * ny);
	const int* src = reinterpret_cast<const int*>(in.data());
	APPFIS::Attribute attr;
	APPFIS::Initialize(argc, argv, APPFIS::DIM_2D, APPFIS::DIM_2D, attr);
	APPFIS::Grid<int> g(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE);
	g.AllocateFullGrid();
	for (int j = 0; j < ny; j++)
		for (int i = 0; i < nx; i++) g.GetFullGrid()->Set(i, j, src[(size_t)j * nx + i]);
	APPFIS::Scatter(g.GetFullGrid(), g.GetSubGrid());
	APPFIS::Config<int> config(g);
	APPFIS::InitializeExecution(g);
	int sm = 0, mx = 0, mn = 0;
	APPFIS::Execute2DReduce(config, sm, APPFIS::SUM, g);
	APPFIS::Execute2DReduce(config, mx, APPFIS::MAX, g);
	APPFIS::Execute2DReduce(config, mn, APPFIS::MIN, g);
	APPFIS::FinalizeExecution(g);
	std::printf("{\"sum\": %d, \"max\": %d, \"min\": %d}\n", sm, mx, mn);
	APPFIS::Finalize();
	return 0;
}

static void GolRun(APPFIS::Config<int>& config, APPFIS::Grid<int>& g, int gens)
{
	for (int t = 0; t < gens; t++) APPFIS::Execute2D(config, g.GetSubGrid(), g.GetSubGridNext());
}

static std::vector<unsigned char> GolInterior(APPFIS::Grid<int>& g, int nx, int ny)
{
	APPFIS::Gather(g.GetFullGrid(), g.GetSubGrid());
	std::vector<unsigned char> out((size_t)nx * ny);
	for (int j = 0; j < ny; j++)
		for (int i = 0; i < nx; i++) out[(size_t)j * nx + i] = (unsigned char)g.GetFullGrid()->Get(i, j);
	return out;
}

static int RunStarPeriodic(int argc, char** argv)
{
	const int nx = std::atoi(argv[2]), ny = std::atoi(argv[3]), nz = std::atoi(argv[4]), iters = std::atoi(argv[5]);
	std::vector<char> in = ReadFile(argv[6], (size_t)nx * ny * nz * sizeof(float));
	const int radius = 4;
	const float coeff = 0.05f;
	APPFIS::Attribute attr;
	attr.ghostLayer = radius;
	attr.periodic = true;
	APPFIS::Initialize(argc, argv, APPFIS::DIM_3D, APPFIS::DIM_3D, attr);
	for (int form = 0; form < 2; form++)
	{
		APPFIS::Grid<float> g(APPFIS::DIM_3D, nx, ny, nz, APPFIS::DUAL);
		g.AllocateFullGrid();
		std::memcpy(g.GetFullGrid()->GetData(), in.data(), in.size());
		APPFIS::Scatter(g.GetFullGrid(), g.GetSubGrid());
		APPFIS::Config<float> config(g);
		config.GridsToUpdate(g);
		APPFIS::InitializeExecution(g);
		for (int t = 0; t < iters; t++)
		{
			if (form == 0) APPFIS::Execute3D(config, coeff, radius, g.GetSubGrid(), g.GetSubGridNext());
			else APPFIS::ExecuteOverlap3D(config, coeff, radius, g.GetSubGrid(), g.GetSubGridNext());
		}
		APPFIS::FinalizeExecution(g);
		APPFIS::Array<float>* sub = g.GetSubGrid();
		WriteFile(argv[7 + form], sub->GetData(), sizeof(float) * (size_t)sub->GetSize());
	}
	std::printf("{\"ok\": true}\n");
	APPFIS::Finalize();
	return 0;
}

// Checkpoint / restart through the device state, and the host binary-file round trip.
static int RunCheckpoint(int argc, char** argv)
{
	const int nx = std::atoi(argv[2]), ny = std::atoi(argv[3]), g1 = std::atoi(argv[4]), g2 = std::atoi(argv[5]);
	std::vector<char> in = ReadFile(argv[6], (size_t)nx * ny);
	const std::string dir(argv[9]);
	const APPFIS::FAST_KERNEL route = Routing(argc, argv, 10, APPFIS::FAST_LIFE);
	APPFIS::Attribute attr;
	attr.ghostLayer = 1;
	attr.periodic = true;
	APPFIS::Initialize(argc, argv, APPFIS::DIM_2D, APPFIS::DIM_2D, attr);
	APPFIS::Grid<int> g(APPFIS::DIM_2D, nx, ny, APPFIS::DUAL), h(APPFIS::DIM_2D, nx, ny, APPFIS::DUAL);
	g.AllocateFullGrid();
	h.AllocateFullGrid();
	for (int j = 0; j < ny; j++)
		for (int i = 0; i < nx; i++) g.GetFullGrid()->Set(i, j, (int)(unsigned char)in[(size_t)j * nx + i]);
	APPFIS::Scatter(g.GetFullGrid(), g.GetSubGrid());
	APPFIS::Config<int> cg(g), ch(h);
	cg.GridsToUpdate(g);
	ch.GridsToUpdate(h);
	APPFIS::UseFastKernel(cg, route);
	APPFIS::UseFastKernel(ch, route);
	APPFIS::InitializeExecution(g, h);
	GolRun(cg, g, g1);
	APPFIS::SaveDeviceState(g, dir + "/state.bin");
	GolRun(cg, g, g2);
	APPFIS::LoadDeviceState(h, dir + "/state.bin");
	GolRun(ch, h, g2);
	APPFIS::FinalizeExecution(g, h);
	std::vector<unsigned char> a = GolInterior(g, nx, ny), b = GolInterior(h, nx, ny);
	WriteFile(argv[7], a.data(), a.size());
	WriteFile(argv[8], b.data(), b.size());
	// host binary files: the gathered grid written and read back
	g.GetFullGrid()->SaveBinaryFile(dir + "/full.bin");
	APPFIS::Array<int> back(APPFIS::DIM_2D, nx, ny);
	back.LoadBinaryFile(dir + "/full.bin");
	bool same = true;
	for (int j = 0; j < ny && same; j++)
		for (int i = 0; i < nx && same; i++) same = back.Get(i, j) == g.GetFullGrid()->Get(i, j);
	std::printf("{\"binary_roundtrip\": %s}\n", same ? "true" : "false");
	APPFIS::Finalize();
	return 0;
}

int main(int argc, char** argv)
{
	if (argc < 2) return 2;
	const std::string mode(argv[1]);
	if (mode == "gol") return RunGol(argc, argv);
	if (mode == "heat2d") return RunHeat2d(argc, argv);
	if (mode == "himeno") return RunHimeno(argc, argv);
	if (mode == "fdtd") return RunFdtd(argc, argv);
	if (mode == "triton") return RunTriton(argc, argv);
	if (mode == "ireduce") return RunIntReduce(argc, argv);
	if (mode == "ckpt") return RunCheckpoint(argc, argv);
	if (mode == "star_periodic") return RunStarPeriodic(argc, argv);
	std::fprintf(stderr, "unknown mode %s\n", argv[1]);
	return 2;
}

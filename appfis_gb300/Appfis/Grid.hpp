/*
 * Grid.hpp — a (possibly double-buffered) field with its ghost ring (reference: Appfis/Grid.hpp).
 *
 * Same interface: GRID_TYPE SINGLE (one buffer, next == current), DUAL (two buffers swapped
 * after each update), FLAT (no ghost ring); GetSubGrid()/GetSubGridNext() return the host
 * arrays before InitializeExecution and descriptors of the device buffers after it
 * (Grid.hpp:295-328); SetBoundary / SetBoundaryCopy fill ghost faces on the host during setup
 * (Grid.hpp:529-830).  The device side is one plain allocation per buffer (no device copy of
 * the Array struct, no dims pointer): kernels get the dims by value.
 */
#ifndef APPFIS_GB_GRID_HPP
#define APPFIS_GB_GRID_HPP

#include <algorithm>
#include <fstream>
#include <string>
#include <vector>

#include "Array.hpp"
#include "Common.hpp"

namespace APPFIS
{

	template<class T>
	class Grid
	{
	private:
		int _nDim = 0;
		int _cur = 0;
		int _next = 0;
		GRID_TYPE _type = SINGLE;
		Array<T> _full;
		Array<T> _host[2];
		T* _dev[2] = { nullptr, nullptr };
		Array<T> _view[2];

	public:
		Grid() {}
		Grid(int nDim, int dimX, GRID_TYPE t) { Create(nDim, dimX, t); }
		Grid(int nDim, int dimX, int dimY, GRID_TYPE t) { Create(nDim, dimX, dimY, t); }
		Grid(int nDim, int dimX, int dimY, int dimZ, GRID_TYPE t) { Create(nDim, dimX, dimY, dimZ, t); }
		Grid(int nDim, int* dims, GRID_TYPE t) { Create(nDim, dims, t); }

		~Grid() { FreeDevice(); }

		Grid(const Grid<T>& o) { CopyHost(o); }

		Grid& operator=(const Grid<T>& o)
		{
			if (this != &o)
			{
				Reset();
				CopyHost(o);
			}
			return *this;
		}

		void Create(int nDim, int dimX, GRID_TYPE t) { Create(nDim, &dimX, t); }
		void Create(int nDim, int dimX, int dimY, GRID_TYPE t)
		{
			int d[2] = { dimX, dimY };
			Create(nDim, d, t);
		}
		void Create(int nDim, int dimX, int dimY, int dimZ, GRID_TYPE t)
		{
			int d[3] = { dimX, dimY, dimZ };
			Create(nDim, d, t);
		}
		void Create(int nDim, int* dims, GRID_TYPE t)
		{
			_nDim = nDim;
			_type = t;
			_full.Resize(nDim, dims);
			CreateSubGrids();
		}

		int GetDimCount() const { return _nDim; }
		GRID_TYPE GetGridType() const { return _type; }
		Array<T>* GetFullGrid() { return &_full; }

		Array<T>* GetSubGrid() { return (ExecutionFlag() && _dev[_cur]) ? &_view[_cur] : &_host[_cur]; }
		Array<T>* GetSubGridNext() { return (ExecutionFlag() && _dev[_next]) ? &_view[_next] : &_host[_next]; }
		Array<T>* GetSubGridCPU() { return &_host[_cur]; }
		Array<T>* GetSubGridNextCPU() { return &_host[_next]; }

		void AllocateFullGrid() { _full.AllocateMemory(); }

		void CreateSubGrids()
		{
			int sub[3] = { 1, 1, 1 };
			if (_type == FLAT)
				for (int a = 0; a < _nDim; a++) sub[a] = _full.GetDim(a);
			else
				GetLocalPartitionDims(_nDim, _full.GetDims(), sub);
			_cur = 0;
			_next = _type == DUAL ? 1 : 0;
			for (int b = 0; b < 2; b++)
			{
				_host[b].Resize(_nDim, sub);
				if (b == 0 || _type == DUAL) _host[b].AllocateMemory();
			}
		}

		// Dirichlet value on every face / one face, in both buffers of a DUAL grid.
		void SetBoundary(T value)
		{
			for (int f = 0; f < 2 * _nDim; f++) SetBoundary(f, value);
		}

		void SetBoundary(int face, T value)
		{
			SetBoundary(&_host[_cur], face, value);
			if (_type == DUAL) SetBoundary(&_host[_next], face, value);
		}

		// Face naming as the reference: 2-D LEFT/RIGHT = x, UP/DOWN = y (UP is the j = 0 side);
		// 3-D LEFT/RIGHT = x, FRONT/BACK = y, DOWN/UP = z (DOWN is the k = 0 side).
		void SetBoundary(Array<T>* arr, int face, T value)
		{
			const int G = GetGhostLayer();
			for (int g = 0; g < G; g++) ForFace(arr, face, g, [&](int i, int j, int k) { Put(arr, i, j, k, value); });
		}

		// Zero-gradient faces: each ghost layer copies its inner neighbour, layers from the inside
		// out (g = G-1 .. 0) with the reference's index arithmetic (Grid.hpp:681-830).
		void SetBoundaryCopy()
		{
			for (int f = 0; f < 2 * _nDim; f++) SetBoundaryCopy(f);
		}

		void SetBoundaryCopy(int face)
		{
			SetBoundaryCopy(&_host[_cur], face);
			if (_type == DUAL) SetBoundaryCopy(&_host[_next], face);
		}

		void SetBoundaryCopy(Array<T>* arr, int face)
		{
			const int G = GetGhostLayer();
			const bool low = (face == LEFT) || (_nDim == 2 ? face == UP : (face == FRONT || face == DOWN));
			const int axis = AxisOf(face);
			for (int g = G - 1; g >= 0; g--)
				ForFace(arr, face, g, [&](int i, int j, int k) {
					int s[3] = { i, j, k };
					s[axis] += low ? 1 : -1;
					Put(arr, i, j, k, Take(arr, s[0], s[1], s[2]));
				});
		}

		void Reset()
		{
			FreeDevice();
			_nDim = 0;
			_full.Reset();
			_host[0].Reset();
			_host[1].Reset();
			_type = SINGLE;
			_cur = _next = 0;
		}

		void Swap() { std::swap(_cur, _next); }

		// ---- engine side
		bool OnDevice() const { return _dev[0] != nullptr; }
		T* DeviceCurrent() { return _dev[_cur]; }
		T* DeviceNext() { return _dev[_next]; }
		int BufferCount() const { return _type == DUAL ? 2 : 1; }

		// Allocates the device buffers (first call) and uploads the host arrays.
		void Upload(cudaStream_t st)
		{
			const size_t bytes = sizeof(T) * (size_t)_host[0].GetSize();
			for (int b = 0; b < BufferCount(); b++)
			{
				if (!_dev[b]) CheckCuda(cudaMalloc((void**)&_dev[b], bytes > 0 ? bytes : sizeof(T)), "cudaMalloc(grid)");
				CheckCuda(cudaMemcpyAsync(_dev[b], _host[b].GetData(), bytes, cudaMemcpyHostToDevice, st), "upload");
				_view[b] = Array<T>(_dev[b], _nDim, _host[b].GetSize(), _host[b].GetDims());
				_view[b].MarkDeviceView();
			}
			if (_type != DUAL)
			{
				_dev[1] = nullptr;
				_view[1] = _view[0];
			}
			CheckCuda(cudaStreamSynchronize(st), "upload");
		}

		// Copies the current device buffer back into its host array (Grid.hpp:471-479).
		void DownloadCurrent(cudaStream_t st)
		{
			if (!_dev[_cur]) return;
			CheckCuda(cudaMemcpyAsync(_host[_cur].GetData(), _dev[_cur], sizeof(T) * (size_t)_host[_cur].GetSize(),
				cudaMemcpyDeviceToHost, st), "download");
			CheckCuda(cudaStreamSynchronize(st), "download");
		}

		bool IsDeviceView(const Array<T>* a) const { return _dev[0] && (a == &_view[0] || a == &_view[1]); }

		// ---- checkpoint of the device state (no counterpart in the reference, whose applications
		// save host arrays after Gather: Array::Save/LoadBinaryFile, Appfis/Array.hpp:421-527).
		// The file holds the padded sub-grid of the current buffer and, for a DUAL grid, the next
		// buffer after it (raw T values, x fastest): both, because a functor may read the next
		// buffer's old values (GameOfLife's stale carry).  Callers run any deferred sweeps first
		// (the engine's SaveDeviceState / LoadDeviceState in Runtime.hpp do).
		bool SaveDevice(const std::string& path, cudaStream_t st)
		{
			if (!_dev[0]) return false;
			const size_t n = (size_t)_host[0].GetSize();
			std::vector<T> buf(n * BufferCount());
			CheckCuda(cudaMemcpyAsync(buf.data(), _dev[_cur], sizeof(T) * n, cudaMemcpyDeviceToHost, st), "checkpoint download");
			if (BufferCount() == 2)
				CheckCuda(cudaMemcpyAsync(buf.data() + n, _dev[_next], sizeof(T) * n, cudaMemcpyDeviceToHost, st), "checkpoint download");
			CheckCuda(cudaStreamSynchronize(st), "checkpoint download");
			CreateDir(GetParentDir(path.c_str()));
			std::ofstream out(path.c_str(), std::ios::binary);
			if (!out.is_open()) return false;
			out.write(reinterpret_cast<const char*>(buf.data()), (std::streamsize)(sizeof(T) * buf.size()));
			return (bool)out;
		}

		bool LoadDevice(const std::string& path, cudaStream_t st)
		{
			if (!_dev[0]) return false;
			const size_t n = (size_t)_host[0].GetSize();
			std::vector<T> buf(n * BufferCount());
			std::ifstream in(path.c_str(), std::ios::binary);
			if (!in.is_open()) return false;
			in.read(reinterpret_cast<char*>(buf.data()), (std::streamsize)(sizeof(T) * buf.size()));
			if (!in) return false;
			CheckCuda(cudaMemcpyAsync(_dev[_cur], buf.data(), sizeof(T) * n, cudaMemcpyHostToDevice, st), "checkpoint upload");
			if (BufferCount() == 2)
				CheckCuda(cudaMemcpyAsync(_dev[_next], buf.data() + n, sizeof(T) * n, cudaMemcpyHostToDevice, st), "checkpoint upload");
			CheckCuda(cudaStreamSynchronize(st), "checkpoint upload");
			return true;
		}

	private:
		void FreeDevice()
		{
			for (int b = 0; b < 2; b++)
			{
				if (_dev[b]) cudaFree(_dev[b]);
				_dev[b] = nullptr;
			}
		}

		void CopyHost(const Grid<T>& o)
		{
			_nDim = o._nDim;
			_type = o._type;
			_cur = o._cur;
			_next = o._next;
			_full = o._full;
			_host[0] = o._host[0];
			_host[1] = o._host[1];
		}

		int AxisOf(int face) const
		{
			if (face == LEFT || face == RIGHT) return 0;
			if (_nDim == 2) return 1;                    // UP / DOWN
			return (face == FRONT || face == BACK) ? 1 : 2;
		}

		static void Put(Array<T>* a, int i, int j, int k, T v)
		{
			if (a->GetDimCount() == 1) a->Set(i, v);
			else if (a->GetDimCount() == 2) a->Set(i, j, v);
			else a->Set(i, j, k, v);
		}

		static T Take(Array<T>* a, int i, int j, int k)
		{
			if (a->GetDimCount() == 1) return a->Get(i);
			if (a->GetDimCount() == 2) return a->Get(i, j);
			return a->Get(i, j, k);
		}

		// Calls fn(i, j, k) for every cell of ghost layer g of `face` (full extent of the other axes).
		template<class F>
		void ForFace(Array<T>* a, int face, int g, F fn)
		{
			const int n = a->GetDimCount();
			const int d[3] = { a->GetDim(0), n > 1 ? a->GetDim(1) : 1, n > 2 ? a->GetDim(2) : 1 };
			if (n == 1 && face != LEFT && face != RIGHT) return;
			if (n == 2 && (face == FRONT || face == BACK)) return;
			const int G = GetGhostLayer();
			const int axis = AxisOf(face);
			const bool low = (face == LEFT) || (n == 2 ? face == UP : (face == FRONT || face == DOWN));
			const int at = low ? g : d[axis] - G + g;
			const int a1 = axis == 0 ? 1 : 0, a2 = axis == 2 ? 1 : 2;
			for (int v = 0; v < d[a2]; v++)
				for (int u = 0; u < d[a1]; u++)
				{
					int c[3];
					c[axis] = at;
					c[a1] = u;
					c[a2] = v;
					fn(c[0], c[1], c[2]);
				}
		}
	};

}

#endif

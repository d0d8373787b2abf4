/*
 * Config.hpp — the iteration box of an Execute call and the grids it updates
 * (reference: Appfis/Config.hpp).  Config(g) covers the interior [ghost, dim - ghost) per axis;
 * the skip constructors cover [skipStart, dim - skipEnd); the raw constructors take the extent
 * directly.  GridsToUpdate(g...) names the grids whose next buffer gets its ghosts refreshed
 * and is swapped in after the sweep.
 */
#ifndef APPFIS_GB_CONFIG_HPP
#define APPFIS_GB_CONFIG_HPP

#include <vector>

#include "Grid.hpp"

namespace APPFIS
{

	template<class T>
	class Config
	{
	private:
		int _dim[3] = { 0, 0, 0 };
		int _start[3] = { 0, 0, 0 };
		int _end[3] = { 0, 0, 0 };

		void Axis(int a, int dim, int s, int e)
		{
			_dim[a] = dim;
			_start[a] = s;
			_end[a] = dim - e;
		}

	public:
		std::vector<Grid<T>*> updatedGrids;

		Config() {}

		explicit Config(Grid<T>& g)
		{
			Array<T>* arr = g.GetSubGridCPU();
			const int G = GetGhostLayer();
			for (int a = 0; a < arr->GetDimCount(); a++) Axis(a, arr->GetDim(a), G, G);
		}

		Config(Grid<T>& g, int sx0, int sx1) { Axis(0, g.GetSubGridCPU()->GetDim(0), sx0, sx1); }

		Config(Grid<T>& g, int sx0, int sx1, int sy0, int sy1)
		{
			Axis(0, g.GetSubGridCPU()->GetDim(0), sx0, sx1);
			Axis(1, g.GetSubGridCPU()->GetDim(1), sy0, sy1);
		}

		Config(Grid<T>& g, int sx0, int sx1, int sy0, int sy1, int sz0, int sz1)
		{
			Axis(0, g.GetSubGridCPU()->GetDim(0), sx0, sx1);
			Axis(1, g.GetSubGridCPU()->GetDim(1), sy0, sy1);
			Axis(2, g.GetSubGridCPU()->GetDim(2), sz0, sz1);
		}

		Config(int dimX, int sx0, int sx1) { Axis(0, dimX, sx0, sx1); }

		Config(int dimX, int sx0, int sx1, int dimY, int sy0, int sy1)
		{
			Axis(0, dimX, sx0, sx1);
			Axis(1, dimY, sy0, sy1);
		}

		Config(int dimX, int sx0, int sx1, int dimY, int sy0, int sy1, int dimZ, int sz0, int sz1)
		{
			Axis(0, dimX, sx0, sx1);
			Axis(1, dimY, sy0, sy1);
			Axis(2, dimZ, sz0, sz1);
		}

		int GetDimX() const { return _dim[0]; }
		int GetDimY() const { return _dim[1]; }
		int GetDimZ() const { return _dim[2]; }
		int GetStartX() const { return _start[0]; }
		int GetStartY() const { return _start[1]; }
		int GetStartZ() const { return _start[2]; }
		int GetEndX() const { return _end[0]; }
		int GetEndY() const { return _end[1]; }
		int GetEndZ() const { return _end[2]; }
		bool IsUpdated() { return !updatedGrids.empty(); }

		void GridsToUpdate(Grid<T>& grid) { updatedGrids.push_back(&grid); }

		template<typename... TArgs>
		void GridsToUpdate(Grid<T>& grid, TArgs&&... args)
		{
			updatedGrids.push_back(&grid);
			GridsToUpdate(args...);
		}
	};

}

#endif

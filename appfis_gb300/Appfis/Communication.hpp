/*
 * Communication.hpp — Scatter / Gather / Exchange / AllReduce of the GB300 APPFIS engine
 * (reference: Appfis/Communication.hpp, MPI).  With one rank:
 *   Scatter(full, sub)  copies the full array into the sub-grid's interior (ghosts untouched),
 *   Gather(full, sub)   copies the sub-grid's interior back into the full array,
 *   AllReduce(v, op)    returns v,
 *   Exchange(arr, ...)  refreshes the periodic ghosts of a HOST array (setup-time use; during
 *                       execution the engine refreshes device ghosts itself).
 * FLAT grids (no ghost ring) copy as a whole.
 */
#ifndef APPFIS_GB_COMMUNICATION_HPP
#define APPFIS_GB_COMMUNICATION_HPP

#include <cstring>
#include <iostream>

#include "Array.hpp"
#include "Common.hpp"

namespace APPFIS
{

	namespace detail
	{
		// Copies between a dense full array and the interior of a padded array (to_sub: full -> sub).
		template<typename T>
		void CopyInterior(Array<T>* full, Array<T>* sub, bool to_sub)
		{
			if (full->GetData() == nullptr || sub->GetData() == nullptr) return;
			const int n = full->GetDimCount();
			const int G = (sub->GetDim(0) == full->GetDim(0)) ? 0 : GetGhostLayer();
			const int fx = full->GetDim(0), fy = n > 1 ? full->GetDim(1) : 1, fz = n > 2 ? full->GetDim(2) : 1;
			const int sx = sub->GetDim(0), sy = n > 1 ? sub->GetDim(1) : 1;
			const int gy = n > 1 ? G : 0, gz = n > 2 ? G : 0;
			T* f = full->GetData();
			T* s = sub->GetData();
			for (int k = 0; k < fz; k++)
				for (int j = 0; j < fy; j++)
				{
					T* fr = f + ((size_t)k * fy + j) * fx;
					T* sr = s + ((size_t)(k + gz) * sy + (j + gy)) * sx + G;
					if (to_sub) std::memcpy(sr, fr, sizeof(T) * fx);
					else std::memcpy(fr, sr, sizeof(T) * fx);
				}
		}
	}

	template<typename T>
	void Scatter(Array<T>* global, Array<T>* local)
	{
		if (global->GetDimCount() != GetDimCount())
		{
			std::cerr << "Partition failed. Data dimension and partition are different." << std::endl;
			std::exit(EXIT_FAILURE);
		}
		detail::CopyInterior(global, local, true);
	}

	template<typename T>
	void Gather(Array<T>* global, Array<T>* local)
	{
		detail::CopyInterior(global, local, false);
	}

	template<typename T>
	T AllReduce(T local, REDUCTION rType)
	{
		(void)rType;
		return local;
	}

	// Periodic ghost refresh of a host array, axis by axis over full faces (the single-rank form
	// of the reference's pack / self-Sendrecv / unpack, Communication.hpp:612-678).
	template<typename T>
	void Exchange(Array<T>* arr)
	{
		const int G = GetGhostLayer();
		if (!IsPeriodic() || G <= 0 || arr->GetData() == nullptr) return;
		const int n = arr->GetDimCount();
		const int d[3] = { arr->GetDim(0), n > 1 ? arr->GetDim(1) : 1, n > 2 ? arr->GetDim(2) : 1 };
		T* f = arr->GetData();
		for (int axis = 0; axis < n; axis++)
		{
			const int a1 = axis == 0 ? 1 : 0, a2 = axis == 2 ? 1 : 2;
			for (int layer = 0; layer < 2 * G; layer++)
			{
				const int dst = layer < G ? layer : d[axis] - G + (layer - G);
				const int src = layer < G ? d[axis] - 2 * G + layer : G + (layer - G);
				for (int v = 0; v < d[a2]; v++)
					for (int u = 0; u < d[a1]; u++)
					{
						int cd[3], cs[3];
						cd[axis] = dst;
						cs[axis] = src;
						cd[a1] = cs[a1] = u;
						cd[a2] = cs[a2] = v;
						f[((size_t)cd[2] * d[1] + cd[1]) * d[0] + cd[0]] = f[((size_t)cs[2] * d[1] + cs[1]) * d[0] + cs[0]];
					}
			}
		}
	}

	template<typename T>
	void ExchangeInitial(Array<T>* arr) { Exchange(arr); }

	inline void ProcessSync()
	{
		if (GetCudaStream()) cudaStreamSynchronize(GetCudaStream());
	}

}

#endif

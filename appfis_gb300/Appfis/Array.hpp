/*
 * Array.hpp — the field container of the GB300 APPFIS engine (reference: Appfis/Array.hpp).
 *
 * Same interface and x-fastest layout as the reference: element (i, j, k) of an array with
 * dims (dX, dY, dZ) lives at i + dX*j + dX*dY*k (Array.hpp:578-589), indices are int.
 * Difference in representation: the dims are stored inside the object (not behind a pointer)
 * and an Array can be a non-owning view of device memory.  The engine hands every kernel a
 * by-value copy of such a view, so Get/Set in a user's Stencil read the dims from registers
 * instead of chasing the reference's device-side `_dims` pointer on every access.
 */
#ifndef APPFIS_GB_ARRAY_HPP
#define APPFIS_GB_ARRAY_HPP

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "Env.hpp"
#include "Utils.hpp"

namespace APPFIS
{

	// What a kernel receives for an Array<T>* argument: a plain copy of the view.
	template<class T>
	struct ArrayArg
	{
		T* data;
		int nDim;
		int size;
		int dims[3];
	};

	template<class T>
	class Array
	{
	private:
		T* _data = nullptr;
		int _nDim = 0;
		int _size = 0;
		int _dims[3] = { 1, 1, 1 };
		bool _owner = false;
		bool _device = false;  // a grid's view of its device buffer (set by Grid::Upload)

	public:
		Array() {}

		Array(int nDim, int dimX) { Shape(nDim, &dimX); }

		Array(int nDim, int dimX, int dimY)
		{
			int d[2] = { dimX, dimY };
			Shape(nDim, d);
		}

		Array(int nDim, int dimX, int dimY, int dimZ)
		{
			int d[3] = { dimX, dimY, dimZ };
			Shape(nDim, d);
		}

		Array(int nDim, int* dims) { Shape(nDim, dims); }

		// Non-owning view (host or device memory).
		EXEC_SPACE Array(T* data, int nDim, int size, const int* dims) : _data(data), _nDim(nDim), _size(size)
		{
			for (int a = 0; a < 3; a++) _dims[a] = dims[a];
		}

		EXEC_SPACE explicit Array(const ArrayArg<T>& v) : _data(v.data), _nDim(v.nDim), _size(v.size)
		{
			for (int a = 0; a < 3; a++) _dims[a] = v.dims[a];
		}

		EXEC_SPACE ~Array()
		{
#if !defined(__CUDA_ARCH__)
			if (_owner && _data) delete[] _data;
#endif
		}

		Array(const Array<T>& o) { CopyFrom(o); }

		Array& operator=(const Array<T>& o)
		{
			if (this != &o)
			{
				Reset();
				CopyFrom(o);
			}
			return *this;
		}

		EXEC_SPACE void Set(int i, T val) { _data[i] = val; }
		EXEC_SPACE void Set(int i, int j, T val) { _data[i + _dims[0] * j] = val; }
		EXEC_SPACE void Set(int i, int j, int k, T val) { _data[i + _dims[0] * j + _dims[0] * _dims[1] * k] = val; }
		EXEC_SPACE T Get(int i) { return _data[i]; }
		EXEC_SPACE T Get(int i, int j) { return _data[i + _dims[0] * j]; }
		EXEC_SPACE T Get(int i, int j, int k) { return _data[i + _dims[0] * j + _dims[0] * _dims[1] * k]; }

		int GetDimCount() const { return _nDim; }
		int GetSize() const { return _size; }
		int GetDim(int dim) const { return _dims[dim]; }
		int* GetDims() const { return const_cast<int*>(_dims); }
		T* GetData() { return _data; }
		bool IsOwner() const { return _owner; }
		bool IsDeviceView() const { return _device; }
		void MarkDeviceView() { _device = true; }

		ArrayArg<T> Arg() const
		{
			ArrayArg<T> a;
			a.data = _data;
			a.nDim = _nDim;
			a.size = _size;
			for (int k = 0; k < 3; k++) a.dims[k] = _dims[k];
			return a;
		}

		void SetData(T* data)
		{
			if (_data == nullptr && _size > 0) AllocateMemory();
			for (int i = 0; i < _size; i++) _data[i] = data[i];
		}

		void FillData(T value)
		{
			if (_data == nullptr && _size > 0) AllocateMemory();
			for (int i = 0; i < _size; i++) _data[i] = value;
		}

		void Square()
		{
			if (_data == nullptr && _size > 0) AllocateMemory();
			for (int i = 0; i < _size; i++) _data[i] = _data[i] * _data[i];
		}

		void Reset()
		{
			if (_owner && _data) delete[] _data;
			_data = nullptr;
			_owner = false;
			_device = false;
			_nDim = 0;
			_size = 0;
			_dims[0] = _dims[1] = _dims[2] = 1;
		}

		// Zero-filled storage, like the reference's `new T[size]()`.
		void AllocateMemory()
		{
			if (_owner && _data) delete[] _data;
			_data = new T[_size > 0 ? _size : 1]();
			_owner = true;
		}

		void Resize(int nDim, int* dims)
		{
			Reset();
			Shape(nDim, dims);
		}

		void LoadAsciiFile(const std::string& filePath, int headerSize = 0)
		{
			std::ifstream in(filePath.c_str());
			if (!in.is_open())
			{
				std::cerr << "Can not read " << filePath << std::endl;
				return;
			}
			if (_data == nullptr && _size > 0) AllocateMemory();
			int index = 0, lineNum = 0;
			std::string line;
			while (std::getline(in, line))
			{
				if (++lineNum <= headerSize) continue;
				StringVector vals = Split(line, ' ');
				for (size_t v = 0; v < vals.size() && index < _size; v++, index++)
					_data[index] = static_cast<T>(std::atof(vals[v].c_str()));
			}
		}

		void LoadBinaryFile(const std::string& filePath, int headerSize = 0)
		{
			std::ifstream in(filePath.c_str(), std::ios::binary);
			if (!in.is_open())
			{
				std::cerr << "Can not read " << filePath << std::endl;
				return;
			}
			if (_data == nullptr && _size > 0) AllocateMemory();
			if (headerSize > 0) in.seekg((std::streamoff)headerSize * sizeof(T), std::ios::beg);
			in.read(reinterpret_cast<char*>(_data), (std::streamsize)sizeof(T) * _size);
		}

		void SaveAsciiFile(const std::string& filePath)
		{
			CreateDir(GetParentDir(filePath.c_str()));
			std::ofstream out(filePath.c_str());
			if (!out.is_open() || _data == nullptr)
			{
				std::cerr << "Can not write to " << filePath << std::endl;
				return;
			}
			out.precision(6);
			out << std::fixed;
			const int dz = _nDim == 3 ? _dims[2] : 1, dy = _nDim >= 2 ? _dims[1] : 1;
			for (int k = 0; k < dz; k++)
				for (int j = 0; j < dy; j++)
				{
					for (int i = 0; i < _dims[0]; i++)
					{
						out << _data[i + _dims[0] * j + _dims[0] * dy * k];
						if (i < _dims[0] - 1) out << " ";
					}
					if (_nDim >= 2) out << "\n";
				}
		}

		void SaveBinaryFile(const std::string& filePath)
		{
			CreateDir(GetParentDir(filePath.c_str()));
			std::ofstream out(filePath.c_str(), std::ios::binary);
			if (!out.is_open() || _data == nullptr)
			{
				std::cerr << "Can not write to " << filePath << std::endl;
				return;
			}
			out.write(reinterpret_cast<const char*>(_data), (std::streamsize)sizeof(T) * _size);
		}

		std::string ToString()
		{
			std::string s;
			if (_data == nullptr) return s;
			const int dz = _nDim == 3 ? _dims[2] : 1, dy = _nDim >= 2 ? _dims[1] : 1;
			bool indent = false;
			for (int k = 0; k < dz; k++)
			{
				for (int j = 0; j < dy; j++)
				{
					if (_nDim == 3 && indent) s += "    ";
					for (int i = 0; i < _dims[0]; i++) s += " " + std::to_string(_data[i + _dims[0] * j + _dims[0] * dy * k]);
					if (_nDim >= 2) s += "\n";
				}
				indent = !indent;
			}
			return s;
		}

	private:
		void Shape(int nDim, const int* dims)
		{
			_nDim = nDim;
			_size = 1;
			for (int a = 0; a < 3; a++) _dims[a] = 1;
			for (int a = 0; a < nDim; a++)
			{
				_dims[a] = dims[a];
				_size *= dims[a];
			}
		}

		void CopyFrom(const Array<T>& o)
		{
			_nDim = o._nDim;
			_size = o._size;
			for (int a = 0; a < 3; a++) _dims[a] = o._dims[a];
			_data = nullptr;
			_owner = false;
			_device = o._device && !o._owner;
			if (o._data != nullptr && o._owner)
			{
				AllocateMemory();
				for (int i = 0; i < _size; i++) _data[i] = o._data[i];
			}
			else
			{
				_data = o._data;  // views stay views
			}
		}
	};

}

#endif

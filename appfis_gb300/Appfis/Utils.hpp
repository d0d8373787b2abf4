/*
 * Utils.hpp — command-line and string/file helpers the applications call, with the reference's
 * signatures (Appfis/Utils.hpp:73-284): CheckArgument / GetArgument parse "-name[=value]"
 * case-insensitively; Split / Trim; CreateDir / GetParentDir for output files.
 */
#ifndef APPFIS_GB_UTILS_HPP
#define APPFIS_GB_UTILS_HPP

#include <sys/stat.h>
#include <sys/types.h>

#include <cctype>
#include <cstdlib>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

namespace APPFIS
{

	namespace detail
	{
		// Argument text after its leading '-' characters.
		inline const char* ArgBody(const char* a)
		{
			while (*a == '-') a++;
			return a;
		}

		inline bool SameNoCase(const char* a, const char* b, size_t n)
		{
			for (size_t i = 0; i < n; i++)
			{
				if (std::tolower((unsigned char)a[i]) != std::tolower((unsigned char)b[i])) return false;
				if (a[i] == '\0') return true;
			}
			return true;
		}
	}

	// True when an argument "-name" or "-name=..." is present (name compared without case).
	inline bool CheckArgument(int argc, char* argv[], const char* name)
	{
		const size_t n = std::strlen(name);
		for (int i = 1; i < argc; i++)
		{
			const char* body = detail::ArgBody(argv[i]);
			const char* eq = std::strchr(body, '=');
			const size_t len = eq ? (size_t)(eq - body) : std::strlen(body);
			if (len == n && detail::SameNoCase(body, name, n)) return true;
		}
		return false;
	}

	// Integer value of "-name=value" (or "-namevalue"); 0 when absent or given without a value.
	inline int GetArgument(int argc, char* argv[], const char* name)
	{
		const size_t n = std::strlen(name);
		bool found = false;
		int value = 0;
		for (int i = 1; i < argc; i++)
		{
			const char* body = detail::ArgBody(argv[i]);
			if (!detail::SameNoCase(body, name, n)) continue;
			found = true;
			if (std::strlen(body) > n) value = std::atoi(body + n + (body[n] == '=' ? 1 : 0));
			else value = 0;
		}
		return found ? value : 0;
	}

	typedef std::vector<std::string> StringVector;

	// Splits on `delim`, keeping empty items (the reference's behaviour, which ASCII field
	// loading depends on).
	inline StringVector& Split(const std::string& s, char delim, StringVector& elems)
	{
		std::stringstream in(s);
		std::string item;
		while (std::getline(in, item, delim)) elems.push_back(item);
		return elems;
	}

	inline StringVector Split(const std::string& s, char delim)
	{
		StringVector elems;
		return Split(s, delim, elems);
	}

	// Each item parsed with operator>> into T (the reference's VecstrToVectype).
	template<typename T>
	std::vector<T> VecstrToVectype(StringVector vs)
	{
		std::vector<T> out;
		for (size_t n = 0; n < vs.size(); n++)
		{
			std::istringstream in(vs[n]);
			T v;
			in >> v;
			out.push_back(v);
		}
		return out;
	}

	// In-place trims returning the argument.
	inline std::string& LeftTrim(std::string& s)
	{
		size_t a = 0;
		while (a < s.size() && std::isspace((unsigned char)s[a])) a++;
		s.erase(0, a);
		return s;
	}

	inline std::string& RightTrim(std::string& s)
	{
		size_t b = s.size();
		while (b > 0 && std::isspace((unsigned char)s[b - 1])) b--;
		s.erase(b);
		return s;
	}

	inline std::string& Trim(std::string& s) { return LeftTrim(RightTrim(s)); }

	inline std::string GetParentDir(const char* path)
	{
		std::string p(path);
		const size_t k = p.find_last_of("/\\");
		return k == std::string::npos ? std::string(".") : p.substr(0, k);
	}

	// Creates `dir` and its missing parents.
	inline void CreateDir(const std::string& dir)
	{
		std::string cur;
		for (size_t i = 0; i <= dir.size(); i++)
		{
			if (i == dir.size() || dir[i] == '/')
			{
				if (!cur.empty() && cur != ".") mkdir(cur.c_str(), 0755);
			}
			if (i < dir.size()) cur += dir[i];
		}
	}

}

#endif

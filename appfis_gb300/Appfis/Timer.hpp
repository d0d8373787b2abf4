/*
 * Timer.hpp — named wall-clock timers (seconds) with the reference's interface
 * (Appfis/Timer.hpp:109-403): Start / Stop / GetCustomTime / GetTotalTime / Reset /
 * CalculateBLUPS (= size * iterations / seconds / 1e9, the GLUP/s the applications print).
 * Category names compare without case, as in the reference.
 *
 * Stop() first waits for the engine's stream, so a timed region covers the GPU work it
 * launched (the reference's GPU build stops its clock with kernels still in flight).
 */
#ifndef APPFIS_GB_TIMER_HPP
#define APPFIS_GB_TIMER_HPP

#include <unistd.h>

#include <algorithm>
#include <cctype>
#include <chrono>
#include <cmath>
#include <ctime>
#include <map>
#include <string>

#include "Common.hpp"

namespace APPFIS
{

	class Timer
	{
	public:
		Timer() {}

		void Start(std::string category)
		{
			if (Context::Get().flushFast) Context::Get().flushFast();  // deferred sweeps belong before the bracket
			_start[Key(category)] = Clock::now();
		}

		void Stop(std::string category)
		{
			if (Context::Get().flushFast) Context::Get().flushFast();  // run the sweeps a fast kernel deferred
			if (Context::Get().stream) cudaStreamSynchronize(Context::Get().stream);
			const std::string k = Key(category);
			std::map<std::string, Clock::time_point>::iterator it = _start.find(k);
			if (it == _start.end()) return;
			_total[k] += std::chrono::duration<double>(Clock::now() - it->second).count();
		}

		void Reset()
		{
			_start.clear();
			_total.clear();
		}

		double GetCustomTime(std::string category)
		{
			std::map<std::string, double>::iterator it = _total.find(Key(category));
			return it == _total.end() ? 0.0 : it->second;
		}

		double GetTotalTime()
		{
			double t = 0.0;
			for (std::map<std::string, double>::iterator it = _total.begin(); it != _total.end(); ++it) t += it->second;
			return t;
		}

		std::string GetCurrentDate()
		{
			char buf[24];
			std::time_t now = std::time(0);
			std::strftime(buf, sizeof buf, "%D", std::localtime(&now));
			return std::string(buf);
		}

		std::string GetHostname()
		{
			char name[1024];
			name[1023] = '\0';
			gethostname(name, 1023);
			return std::string(name);
		}

		int AddNewTimer(std::string category)
		{
			const std::string k = Key(category);
			if (_total.find(k) == _total.end()) _total[k] = 0.0;
			return (int)std::distance(_total.begin(), _total.find(k));
		}

		double CalculateBLUPS(std::string category, int size, int iter)
		{
			const double t = GetCustomTime(category);
			return ((double)size * iter) / (t * std::pow(10, 9));
		}

	private:
		typedef std::chrono::steady_clock Clock;
		std::map<std::string, Clock::time_point> _start;
		std::map<std::string, double> _total;

		static std::string Key(std::string s)
		{
			std::transform(s.begin(), s.end(), s.begin(), [](unsigned char c) { return (char)std::tolower(c); });
			return s;
		}
	};

}

#endif

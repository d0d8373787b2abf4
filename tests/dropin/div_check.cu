// Host check of the drop-in executors' multiply-shift division (Appfis/Runtime.hpp MakeDiv /
// DivQ, used to number ragged planes): exact quotients over a spread of divisors and numerators
// below 2^31, the range those launches use.  Prints "ok" and exits 0, or names the first failure.
#define APPFIS_CUDA 1
#include "Appfis/Appfis.hpp"

#include <cstdio>

int main()
{
    unsigned long long x = 0x9e3779b97f4a7c15ull, checks = 0;
    auto next = [&]() { x ^= x << 13; x ^= x >> 7; x ^= x << 17; return x; };
    for (int t = 0; t < 40000; t++)
    {
        const int d = t < 5000 ? t + 1 : (int)(next() % 0x7fffffffull) + 1;
        const APPFIS::detail::Div v = APPFIS::detail::MakeDiv(d);
        const unsigned ns[] = { 0u, 1u, (unsigned)d - 1, (unsigned)d, 0x7fffffffu, 0x7ffffffeu, (unsigned)(next() & 0x7fffffffu),
            (unsigned)(((0x7fffffffull / (unsigned)d) * (unsigned)d) - 1), (unsigned)((0x7fffffffull / (unsigned)d) * (unsigned)d) };
        for (unsigned n : ns)
        {
            if (n > 0x7fffffffu) continue;
            const unsigned q = APPFIS::detail::DivQ(n, v);
            checks++;
            if (q != n / (unsigned)d)
            {
                std::printf("FAIL d=%d n=%u q=%u\n", d, n, q);
                return 1;
            }
        }
    }
    std::printf("ok %llu\n", checks);
    return 0;
}

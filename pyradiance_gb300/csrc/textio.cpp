/*
 * textio.cpp -- ASCII output of the drop-in programs: rows of numbers in
 * C's %e form (six digits after the point), the form rtrace and rcontrib
 * print values in (rt/rtrace.c puta, rt/rc2.c), formatted by several host
 * threads.  Each thread formats a contiguous range of rows into its own
 * buffer; the buffers are then joined in row order, so the text equals a
 * single-threaded loop's.
 */
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gbrad.h"

extern "C" int gb_format_rows(const double *vals, int64_t nrows, int64_t ncols, const char *sep, const char *end,
                              char *out, int64_t cap, int64_t *len)
{
    if (nrows < 0 || ncols < 0 || (nrows > 0 && ncols > 0 && !vals) || !sep || !end || !len || (cap > 0 && !out))
        return GB_EINVAL;
    const size_t lsep = strlen(sep), lend = strlen(end);
    int nt = (int)std::max(1u, std::thread::hardware_concurrency());
    if ((int64_t)nt > nrows / 256 + 1)
        nt = (int)(nrows / 256 + 1);
    std::vector<std::string> part((size_t)nt);
    auto work = [&](int t) {
        const int64_t r0 = nrows * t / nt, r1 = nrows * (t + 1) / nt;
        std::string &s = part[(size_t)t];
        s.reserve((size_t)((r1 - r0) * (ncols * (16 + (int64_t)lsep) + (int64_t)lend)));
        char buf[64];
        for (int64_t r = r0; r < r1; r++) {
            const double *v = vals + r * ncols;
            for (int64_t c = 0; c < ncols; c++) {
                const int n = snprintf(buf, sizeof buf, "%e", v[c]);
                s.append(buf, (size_t)n);
                if (c + 1 < ncols)
                    s.append(sep, lsep);
            }
            s.append(end, lend);
        }
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nt; t++)
        th.emplace_back(work, t);
    work(0);
    for (auto &x : th)
        x.join();
    int64_t total = 0;
    for (const auto &s : part)
        total += (int64_t)s.size();
    *len = total;
    if (total > cap)
        return GB_EOVERFLOW;
    char *p = out;
    for (const auto &s : part) {
        memcpy(p, s.data(), s.size());
        p += s.size();
    }
    return GB_OK;
}

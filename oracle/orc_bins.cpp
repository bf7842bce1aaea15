/*
 * orc_bins.cpp -- TEST INFRASTRUCTURE: C-callable wrapper that lets the CPU
 * oracle compile rcontrib bin expressions with the library's host compiler
 * (pyradiance_gb300/csrc/binexpr.cpp), so both evaluate the same program.
 */
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../include/gbrad.h"
#include "../pyradiance_gb300/csrc/binexpr.h"

extern "C" int orc_compile_bins(const gb_modspec *mods, int nmods, gb_binins *prog, int progcap, int *info,
                                int *nbt, char *err, int errlen)
{
    int total = 0, used = 0;
    for (int m = 0; m < nmods; m++) {
        std::vector<gb_binins> p;
        std::string e;
        int nb = 0;
        if (gb_compile_bin(mods[m].binv, mods[m].params, mods[m].calfile, mods[m].expr, mods[m].nbins, p, &nb,
                           e) < 0) {
            snprintf(err, errlen, "modifier '%s': %s", mods[m].modifier, e.c_str());
            return -1;
        }
        if (used + (int)p.size() > progcap) {
            snprintf(err, errlen, "bin programs too long");
            return -1;
        }
        memcpy(prog + used, p.data(), p.size() * sizeof(gb_binins));
        info[3 * m] = used;
        info[3 * m + 1] = nb;
        info[3 * m + 2] = total;
        used += (int)p.size();
        total += nb;
    }
    *nbt = total;
    return 0;
}

extern "C" int orc_nbins(const gb_modspec *mods, int nmods, char *err, int errlen)
{
    static thread_local gb_binins prog[4096];
    int info[3 * 256], nbt = 0;
    if (nmods > 256 || orc_compile_bins(mods, nmods, prog, 4096, info, &nbt, err, errlen) < 0)
        return -1;
    return nbt;
}

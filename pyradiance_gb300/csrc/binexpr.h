/* binexpr.h -- host compiler of rcontrib bin expressions (binexpr.cpp) */
#ifndef GB_BINEXPR_H
#define GB_BINEXPR_H

#include <string>
#include <vector>
#include "gbcommon.h"

/* Compile binv (with -p params, -f calfile, -e definitions) into a device
 * program; *nbins is the -bn count on input (0 if none) and the final count
 * on output; nbins_expr, when given, is the -bn text evaluated with the same
 * definitions.  Returns 0, or -1 with err set. */
int gb_compile_bin(const char *binv, const char *params, const char *calfile, const char *expr,
                   const char *nbins_expr, std::vector<gb_binins> &prog, int *nbins, std::string &err);

double reinhart_nbins(double MF);

#endif

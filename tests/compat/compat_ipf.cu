// Quadrature-file handling of the drop-in headers (host only): prints
// "builtin", "rules <nq> <nqs>" or "error <message>" for the IPF.txt /
// IPFs.txt found in the current directory.
#include <cstdio>
#include <stdexcept>
#include "ibem.cuh"

int main()
{
    std::vector<double> reg, sing;
    ia_rules rules;
    try {
        const ia_rules *r = ia_compat_rules(reg, sing, rules, "ibem");
        if (!r) std::printf("builtin\n");
        else std::printf("rules %d %d\n", r->nq, r->nqs);
    } catch (const std::runtime_error &e) {
        std::printf("error %s\n", e.what());
    }
    return 0;
}

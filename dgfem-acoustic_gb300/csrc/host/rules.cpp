#include "rules.h"

namespace dg {
namespace {
#include "rules.inc"
}

QuadRule quad_rule(int dim, int degree) {
    const double *t = nullptr;
    int n = 0;
#define DG_RULE(D, DEG, NAME) \
    if (dim == D && degree == DEG) { t = NAME; n = NAME##_n; }
    DG_RULE(1, 2, kRuleLine2) DG_RULE(1, 4, kRuleLine4) DG_RULE(1, 6, kRuleLine6)
    DG_RULE(1, 8, kRuleLine8) DG_RULE(1, 10, kRuleLine10)
    DG_RULE(2, 2, kRuleTri2) DG_RULE(2, 4, kRuleTri4) DG_RULE(2, 6, kRuleTri6)
    DG_RULE(2, 8, kRuleTri8) DG_RULE(2, 10, kRuleTri10)
    DG_RULE(3, 2, kRuleTet2) DG_RULE(3, 4, kRuleTet4) DG_RULE(3, 6, kRuleTet6)
    DG_RULE(3, 8, kRuleTet8) DG_RULE(3, 10, kRuleTet10)
#undef DG_RULE
    QuadRule r;
    if (!t) return r;
    r.n = n;
    r.uvwq.assign(t, t + 4 * n);
    return r;
}

}  // namespace dg

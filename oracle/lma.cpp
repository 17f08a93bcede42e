// Oracle (test infrastructure only): see lma.h.
#include "lma.h"

namespace orc {

int lma_radiate(const Laser&, const V4&, const V4&, double, DrawStream&, bool, bool* emitted, RadiationEvent*,
                uint64_t*) {
    *emitted = false;
    return PTG_ERR_UNSUPPORTED;
}

int lma_pair_create(const Laser&, const V4&, const V4&, const Stokes& pol, double, DrawStream&, double, double* prob,
                    Stokes* pol_new, bool* created, PairEvent*, uint64_t*) {
    *prob = 0.0;
    *pol_new = pol;
    *created = false;
    return PTG_ERR_UNSUPPORTED;
}

}  // namespace orc

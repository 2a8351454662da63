/* p8est_bits.h: covered by p4est_to_p8est.h in this shim. */
#include "p4est_to_p8est.h"

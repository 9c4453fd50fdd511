/* Test infrastructure: the one out-of-line definition the shimmed reference build needs. */
#include "oic_ref_shim.H"

sqStore *ovOverlap::g = NULL;

/* types.H -- test infrastructure only: the meryl-utility header canu names, served by ovs_shim.H. */
#include "ovs_shim.H"

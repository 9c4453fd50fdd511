/* Shim header for compiling canu overlapInCore sources as the CPU reference (oracle/_ref). */
#include "oic_ref_shim.H"

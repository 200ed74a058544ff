/* Arch header name used by the reference host sources (main.c, flow_data.c,
 * flow_interface.h); for the GB300 kernel set everything lives in
 * flow_arch.h and flow_gb300.h. */
#include "../flow_arch.h"
#include "../flow_gb300.h"

/* ORACLE TEST INFRASTRUCTURE: arch header name used by the reference sources;
 * everything lives in arch_shim.h. */
#include "arch_shim.h"

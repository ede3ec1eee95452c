/*
 * TEST INFRASTRUCTURE ONLY -- the FP64 port of afft (port64_*): the same
 * algorithm on doubles, as afft's afft_64_* entry points run it.
 */
typedef double preal;
#define PORT(name) port64_##name
#define PORT_SIN sin
#define PORT_COS cos
#define PORT_LDEXP ldexp
#include "afft_port.inc"

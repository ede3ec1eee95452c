/*
 * TEST INFRASTRUCTURE ONLY -- the FP32 port of afft (port32_*).
 */
typedef float preal;
#define PORT(name) port32_##name
#define PORT_SIN sinf
#define PORT_COS cosf
#define PORT_LDEXP ldexpf
#include "afft_port.inc"

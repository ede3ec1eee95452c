/* Stand-in for afft's fft.h: the reference's own C++ wrapper (fft.hpp)
 * includes "fft.h"; this forwards it to the GB300 library's header, which
 * declares the same entry points (include/afft_gb300.h). */
#include "../../include/afft_gb300.h"

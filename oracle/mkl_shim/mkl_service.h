/* MKL-API shim (oracle test infrastructure): everything lives in mkl.h. */
#include "mkl.h"

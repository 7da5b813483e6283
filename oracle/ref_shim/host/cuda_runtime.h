/* host emulation stand-in: see gb_host_cuda.h (test infrastructure only) */
#pragma once
#include "gb_host_cuda.h"

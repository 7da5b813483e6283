/* host emulation stand-in: see gb_host_libs.h (test infrastructure only) */
#pragma once
#include "gb_host_libs.h"

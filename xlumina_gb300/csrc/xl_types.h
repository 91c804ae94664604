// Types shared by the C ABI and the device code.
#pragma once
#include "xlgb.h"

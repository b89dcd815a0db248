// Project-written stand-in: everything lives in tbb.h.
#pragma once
#include "tbb.h"

// Stand-in header: every name the reference uses lives in ddshim_common.hpp.
#pragma once
#include "ddshim_common.hpp"

// Project-written stand-in (test infrastructure).  RandBLAS includes this header
// (RandBLAS/random_gen.hh:38) but its sketching path only uses Philox4x32.
#pragma once
#include "array.h"

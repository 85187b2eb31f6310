// The reference includes "Cell.hpp"; its tree holds the header as Cell.cuh.
#pragma once
#include "Cell.cuh"

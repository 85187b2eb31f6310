// The reference includes "MD.hpp"; its tree holds the header as MD.cuh.
#pragma once
#include "MD.cuh"

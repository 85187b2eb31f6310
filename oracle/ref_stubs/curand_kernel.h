// Stand-in: MD.cuh names curandState in declarations of its (uncompiled) device draft.
#pragma once
struct curandState {};

// Stand-in for the one Boost header the reference's Utils.hpp includes but whose contents the
// compiled parts (BoundingBox, Nint, LinkListOrtho) do not use. Test infrastructure only:
// lets oracle/ref_build.sh compile those parts from the reference tree without Boost.
#pragma once

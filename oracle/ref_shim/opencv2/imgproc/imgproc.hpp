// Stand-in: painty's Serialization.cxx includes this OpenCV header; the parts it uses are in
// the repository stand-in opencv2/imgproc.hpp.
#pragma once
#include "opencv2/imgproc.hpp"

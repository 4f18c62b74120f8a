// Stand-in: OpenCV core, as far as the repository stand-in in imgproc.hpp goes.
#pragma once
#include "opencv2/imgproc.hpp"

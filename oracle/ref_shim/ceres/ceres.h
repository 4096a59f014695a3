#include <ceres/jet.h>

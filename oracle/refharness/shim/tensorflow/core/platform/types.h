// Stand-in for TensorFlow's platform types header (nothing from it is used).
#pragma once
#include <cstdint>

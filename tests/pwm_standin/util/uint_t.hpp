// Stand-in for pwm's util/uint_t.hpp (test infrastructure only).
#pragma once
#include "util/type_for_bytes.hpp"

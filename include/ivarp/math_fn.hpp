// Expression API used by lemma definitions (the reference's ivarp/math_fn.hpp).
#pragma once

#include <iostream>
#include <sstream>
#include <string>

#include "sid_fe/types.hpp"
#include "sid_fe/expr.hpp"

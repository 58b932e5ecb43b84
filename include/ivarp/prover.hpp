// Variables, constraint systems and prover inputs (the reference's ivarp/prover.hpp).
#pragma once

#include "math_fn.hpp"
#include "sid_fe/api.hpp"

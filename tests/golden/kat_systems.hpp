// Known-answer constraint systems for the prover tests, written against the ivarp front end.
// They re-express the scenarios of the reference's prover tests:
//   expected_critical   : ivarp/test/expected_criticals.cpp:46-96 (2 vars, dyn(8,2) + 4, 2 generations)
//   expected_critical2  : ivarp/test/expected_criticals2.cpp:33-43 (4 vars, dyn(4,4) x2 + 8 + 8)
//   pos_neg1_sat/unsat  : ivarp/test/positive_and_negative_proof1.cpp:31-43 (dyn(8,4) + 64)
//   pos_neg2_sat/unsat  : ivarp/test/positive_and_negative_proof2.cpp:36-55 (dyn(8,4) x2 + 128 + 128)
//   run_prover_sat/unsat: ivarp/test/run_prover.cpp:29-40 (dyn(64,2) + 32)
// Used by kat_systems.cpp (writes their IR for the GPU build) and tests/run_prover_gpu.cpp (proves them on
// the GPU through ivarp::run_prover).
#pragma once

#include <ivarp/run_prover.hpp>

namespace kat {

using namespace ivarp;
using namespace ivarp::args;

/// Calls visit(name, constraint system, prover input) for every system, in the order of the IR file names
/// of make_kat_ir.py.
template<typename Visit> void for_each_system(Visit&& visit) {
    {
        const auto x = x0;
        const auto y = x1;
        const auto cs = constraint_system(variable(x, "x", 0_Z, 2_Z), variable(y, "y", 0_Z, 2_Z),
                                          x >= y, x <= 3_Z - y, y <= 3_Z - x);
        using Split = U64Pack<dynamic_subdivision(8, 2), 4>;
        visit("expected_critical_f64", cs, prover_input<DefaultContextWithNumberType<IDouble>, Split>(cs));
        visit("expected_critical_f32", cs, prover_input<DefaultContextWithNumberType<IFloat>, Split>(cs));
    }
    {
        const auto w = x0, x = x1, y = x2, z = x3;
        const auto cs = constraint_system(variable(w, "w", 0_Z, 1_Z), variable(x, "x", 0_Z, 1_Z),
                                          variable(y, "y", 0_Z, 1_Z), variable(z, "z", 0_Z, 1_Z),
                                          w + x + y + z >= 0);
        using Split = U64Pack<dynamic_subdivision(4, 4), dynamic_subdivision(4, 4), 8, 8>;
        visit("expected_critical2_f64", cs, prover_input<DefaultContextWithNumberType<IDouble>, Split>(cs));
        visit("expected_critical2_f32", cs, prover_input<DefaultContextWithNumberType<IFloat>, Split>(cs));
    }
    {
        const auto x = x0, y = x1;
        const auto f = fixed_pow<3>(x) - 2 * square(y) - 3 * x + sqrt(y);
        const auto sat = constraint_system(variable(x, "x", -2_Z, 2_Z), variable(y, "y", 0_Z, 2_Z), f > 2.37_X, y >= x);
        const auto unsat = constraint_system(variable(x, "x", -2_Z, 2_Z), variable(y, "y", 0_Z, 2_Z), f > 2.38_X, y >= x);
        using Split = U64Pack<dynamic_subdivision(8, 4), 64>;
        visit("pos_neg1_sat", sat, prover_input<DefaultContextWithNumberType<IDouble>, Split>(sat));
        visit("pos_neg1_unsat", unsat, prover_input<DefaultContextWithNumberType<IDouble>, Split>(unsat));
    }
    {
        const auto w = x0, x = x1, y = x2, z = x3;
        const auto f = -w * (fixed_pow<3>(x) - 2_Z * square(y) + sqrt(y)) + w / z;
        const auto unsat = constraint_system(variable(w, "w", -2_Z, 2_Z), variable(x, "x", -2_Z, 2_Z),
                                             variable(y, "y", 0_Z, 5_Z), variable(z, "z", 0.5_X, 8_Z),
                                             f > 111.927865_X, x <= w, z >= y);
        const auto sat = constraint_system(variable(w, "w", -2_Z, 2_Z), variable(x, "x", -2_Z, 2_Z),
                                           variable(y, "y", 0_Z, 5_Z), variable(z, "z", 0.5_X, 8_Z),
                                           f > 111.927864_X, x <= w, z >= y);
        using Split = U64Pack<dynamic_subdivision(8, 4), dynamic_subdivision(8, 4), 128, 128>;
        visit("pos_neg2_sat", sat, prover_input<DefaultContextWithNumberType<IDouble>, Split>(sat));
        visit("pos_neg2_unsat", unsat, prover_input<DefaultContextWithNumberType<IDouble>, Split>(unsat));
    }
    {
        const auto x = x0, y = x1;
        const auto cube = fixed_pow<3>(x0);
        const auto f = cube(x) - 2_Z * square(y) - 3_Z * x + sqrt(y);
        const auto sat = constraint_system(variable(x, "x", -2_Z, 2_Z), variable(y, "y", 0, 2), y >= x, f >= 2.37_X);
        const auto unsat = constraint_system(variable(x, "x", -2_Z, 2_Z), variable(y, "y", 0, 2), y >= x, f >= 2.38_X);
        using Split = U64Pack<dynamic_subdivision(64, 2), 32>;
        visit("run_prover_sat_f64", sat, prover_input<DefaultContextWithNumberType<IDouble>, Split>(sat));
        visit("run_prover_unsat_f64", unsat, prover_input<DefaultContextWithNumberType<IDouble>, Split>(unsat));
        visit("run_prover_sat_f32", sat, prover_input<DefaultContextWithNumberType<IFloat>, Split>(sat));
        visit("run_prover_unsat_f32", unsat, prover_input<DefaultContextWithNumberType<IFloat>, Split>(unsat));
    }
}

} // namespace kat

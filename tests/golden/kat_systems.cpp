// Known-answer constraint systems for the prover tests, written against the ivarp front end.
// They re-express the scenarios of the reference's prover tests:
//   expected_critical   : ivarp/test/expected_criticals.cpp:46-96 (2 vars, dyn(8,2) + 4, 2 generations)
//   expected_critical2  : ivarp/test/expected_criticals2.cpp:33-43 (4 vars, dyn(4,4) x2 + 8 + 8)
//   pos_neg1_sat/unsat  : ivarp/test/positive_and_negative_proof1.cpp:31-43 (dyn(8,4) + 64)
//   pos_neg2_sat/unsat  : ivarp/test/positive_and_negative_proof2.cpp:36-55 (dyn(8,4) x2 + 128 + 128)
//   run_prover_sat/unsat: ivarp/test/run_prover.cpp:29-40 (dyn(64,2) + 32)
// Built and run by make_kat_ir.py with SID_EXPORT_DIR set: every run_prover call writes its IR.
#include <ivarp/run_prover.hpp>

using namespace ivarp;
using namespace ivarp::args;

template<typename Input> static void emit(const Input& in) {
    run_prover(in, [](const auto&, const auto*) {});
}

int main() {
    {
        const auto x = x0;
        const auto y = x1;
        const auto cs = constraint_system(variable(x, "x", 0_Z, 2_Z), variable(y, "y", 0_Z, 2_Z),
                                          x >= y, x <= 3_Z - y, y <= 3_Z - x);
        using Split = U64Pack<dynamic_subdivision(8, 2), 4>;
        emit(prover_input<DefaultContextWithNumberType<IDouble>, Split>(cs));
        emit(prover_input<DefaultContextWithNumberType<IFloat>, Split>(cs));
    }
    {
        const auto w = x0, x = x1, y = x2, z = x3;
        const auto cs = constraint_system(variable(w, "w", 0_Z, 1_Z), variable(x, "x", 0_Z, 1_Z),
                                          variable(y, "y", 0_Z, 1_Z), variable(z, "z", 0_Z, 1_Z),
                                          w + x + y + z >= 0);
        using Split = U64Pack<dynamic_subdivision(4, 4), dynamic_subdivision(4, 4), 8, 8>;
        emit(prover_input<DefaultContextWithNumberType<IDouble>, Split>(cs));
        emit(prover_input<DefaultContextWithNumberType<IFloat>, Split>(cs));
    }
    {
        const auto x = x0, y = x1;
        const auto f = fixed_pow<3>(x) - 2 * square(y) - 3 * x + sqrt(y);
        const auto sat = constraint_system(variable(x, "x", -2_Z, 2_Z), variable(y, "y", 0_Z, 2_Z), f > 2.37_X, y >= x);
        const auto unsat = constraint_system(variable(x, "x", -2_Z, 2_Z), variable(y, "y", 0_Z, 2_Z), f > 2.38_X, y >= x);
        using Split = U64Pack<dynamic_subdivision(8, 4), 64>;
        emit(prover_input<DefaultContextWithNumberType<IDouble>, Split>(sat));
        emit(prover_input<DefaultContextWithNumberType<IDouble>, Split>(unsat));
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
        emit(prover_input<DefaultContextWithNumberType<IDouble>, Split>(sat));
        emit(prover_input<DefaultContextWithNumberType<IDouble>, Split>(unsat));
    }
    {
        const auto x = x0, y = x1;
        const auto cube = fixed_pow<3>(x0);
        const auto f = cube(x) - 2_Z * square(y) - 3_Z * x + sqrt(y);
        const auto sat = constraint_system(variable(x, "x", -2_Z, 2_Z), variable(y, "y", 0, 2), y >= x, f >= 2.37_X);
        const auto unsat = constraint_system(variable(x, "x", -2_Z, 2_Z), variable(y, "y", 0, 2), y >= x, f >= 2.38_X);
        using Split = U64Pack<dynamic_subdivision(64, 2), 32>;
        emit(prover_input<DefaultContextWithNumberType<IDouble>, Split>(sat));
        emit(prover_input<DefaultContextWithNumberType<IDouble>, Split>(unsat));
        emit(prover_input<DefaultContextWithNumberType<IFloat>, Split>(sat));
        emit(prover_input<DefaultContextWithNumberType<IFloat>, Split>(unsat));
    }
    return 0;
}

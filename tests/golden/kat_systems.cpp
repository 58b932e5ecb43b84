// Writes the IR of the known-answer systems (kat_systems.hpp): built and run by make_kat_ir.py with
// SID_EXPORT_DIR set, so every run_prover call writes its compiled IR instead of proving.
#include "kat_systems.hpp"

int main() {
    kat::for_each_system([](const char*, const auto&, const auto& input) {
        ivarp::run_prover(input, [](const auto&, const auto*) {});
    });
    return 0;
}

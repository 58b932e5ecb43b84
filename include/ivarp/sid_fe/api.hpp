// Constraint systems, variables and prover inputs (the reference's
// variable_description.hpp, constraint_system.hpp:82-95 and prover_input.hpp:118-122).
#pragma once

#include <memory>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "compile.hpp"

namespace ivarp {

/// Looks up variable names by argument index (used by the printers).
class ArgNameLookup {
public:
    virtual ~ArgNameLookup() = default;
    virtual std::string arg_name(std::size_t arg_index) const = 0;
};

/// A variable with its symbolic lower and upper bound (variable_description.hpp:30-110).
struct VariableDescription {
    int index;
    std::string name;
    sid_fe::NP lb, ub;
    bool is_value = false;
};

template<typename StringArg, typename LBT, typename UBT,
         std::enable_if_t<sid_fe::IsExprLike<LBT>::value && sid_fe::IsExprLike<UBT>::value, int> = 0>
inline VariableDescription variable(const MathExpr& arg, StringArg&& name, const LBT& lb, const UBT& ub) {
    if(arg.get()->op != sid_fe::Op::Arg) throw std::invalid_argument("variable() needs an argument placeholder");
    return VariableDescription{arg.get()->arg, std::string(std::forward<StringArg>(name)),
                               sid_fe::to_node(lb), sid_fe::to_node(ub)};
}

/// A value defined by an expression of earlier variables (`value(x, expr, name)`): it is treated as a
/// variable whose bounds are given by the constraint x == expr.
template<typename StringArg, typename E, std::enable_if_t<sid_fe::IsExprLike<E>::value, int> = 0>
inline VariableDescription value(const MathExpr& arg, const E& expr, StringArg&& name) {
    if(arg.get()->op != sid_fe::Op::Arg) throw std::invalid_argument("value() needs an argument placeholder");
    auto e = sid_fe::to_node(expr);
    return VariableDescription{arg.get()->arg, std::string(std::forward<StringArg>(name)), e, e, true};
}

/// Variables plus constraints. Variable bounds become the first constraints, in the order the
/// variables were given (constraint_system/extract_bound_constraints.hpp:30-53).
class ConstraintSystem : public ArgNameLookup {
public:
    std::vector<sid_fe::VarDesc> vars;
    std::vector<sid_fe::NP> constraints;

    std::size_t num_args() const noexcept { return vars.size(); }

    std::string arg_name(std::size_t arg_index) const override {
        for(const auto& v : vars) if(std::size_t(v.arg) == arg_index) return v.name;
        throw std::out_of_range("arg_index out of range in ConstraintSystem::arg_name!");
    }
};

namespace sid_fe {
inline void add_to_system(ConstraintSystem& cs, const VariableDescription& v) {
    cs.vars.push_back(VarDesc{v.index, v.name, v.lb, v.ub, v.is_value});
}
inline void add_to_system(ConstraintSystem& cs, const MathPred& p) { cs.constraints.push_back(p.get()); }
inline void add_to_system(ConstraintSystem& cs, bool b) { cs.constraints.push_back(make_bool_const(b, b)); }
} // namespace sid_fe

template<typename... Items> inline ConstraintSystem constraint_system(const Items&... items) {
    ConstraintSystem cs;
    int dummy[] = {0, (sid_fe::add_to_system(cs, items), 0)...};
    (void)dummy;
    return cs;
}

namespace sid_fe {
template<typename NT> struct NumberTypeName;
template<> struct NumberTypeName<IDouble> { static const char* get() { return "f64"; } };
template<> struct NumberTypeName<IFloat> { static const char* get() { return "f32"; } };
} // namespace sid_fe

/// A compiled constraint system with its split configuration, ready for run_prover.
template<typename Context_> struct ProverInput {
    using Context = Context_;
    using NumberType = typename Context::NumberType;

    std::shared_ptr<const sid_fe::CompiledLemma> lemma;
    std::string ir;                       ///< text IR consumed by the engine
    std::shared_ptr<const ConstraintSystem> system;

    std::size_t num_args() const noexcept { return std::size_t(lemma->nargs); }
};

/// Compile a constraint system (the reference's prover_input<Context, U64Pack<...>>(system)).
template<typename Context, typename VariableSplitting>
inline ProverInput<Context> prover_input(const ConstraintSystem& system) {
    using NT = typename Context::NumberType;
    auto lemma = std::make_shared<sid_fe::CompiledLemma>(
        sid_fe::compile_system(system.vars, system.constraints, VariableSplitting::values(),
                               sid_fe::NumberTypeName<NT>::get()));
    ProverInput<Context> in;
    in.ir = sid_fe::to_ir(*lemma);
    in.lemma = lemma;
    in.system = std::make_shared<const ConstraintSystem>(system);
    return in;
}

} // namespace ivarp

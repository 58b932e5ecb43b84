// Critical-cuboid printer (the reference's ivarp/critical_printer.hpp:27-110).
#pragma once

#include <mutex>
#include <ostream>
#include <sstream>
#include <string>
#include <tuple>
#include <utility>

#include "prover.hpp"
#include "sid_fe/host_eval.hpp"

namespace ivarp {

/// An expression printed next to each critical cuboid.
template<typename ExpressionType> struct PrintExpr {
    template<typename S, typename E> PrintExpr(S&& n, E&& e) : name(std::forward<S>(n)), expr(std::forward<E>(e)) {}
    std::string name;
    ExpressionType expr;
};

template<typename StringArg, typename EType> inline auto printable_expression(StringArg&& name, EType&& expr) {
    return PrintExpr<std::decay_t<EType>>{std::forward<StringArg>(name), std::forward<EType>(expr)};
}

/// Prints every critical cuboid: one line per variable, then one line per printable expression with its
/// interval value on the cuboid (evaluated on the host by sid_fe::HostEvaluator).
template<bool Locking, typename... OutputExprs> class CriticalPrinter {
public:
    CriticalPrinter(const ArgNameLookup* lookup, std::size_t num_args, std::ostream* output, OutputExprs... exprs) :
        name_lookup(lookup), num_args(num_args), output(output), exprs(std::move(exprs)...),
        evaluators(std::make_shared<std::vector<sid_fe::HostEvaluator>>()) {
        make_evaluators(std::index_sequence_for<OutputExprs...>{});
    }

    template<typename Context, typename ValueArray> void operator()(const Context&, const ValueArray& values) const {
        std::ostringstream out;
        out << "Critical:\n";
        for(std::size_t i = 0; i < num_args; ++i) {
            out << '\t' << name_lookup->arg_name(i) << ": " << values[i] << std::endl;
        }
        std::vector<IDouble> box(num_args);
        for(std::size_t i = 0; i < num_args; ++i) box[i] = IDouble(values[i].lb(), values[i].ub(), values[i].possibly_undefined());
        print_values(out, box.data(), std::index_sequence_for<OutputExprs...>{});
        std::unique_lock<std::mutex> lock(*mtx, std::defer_lock);
        if(Locking) lock.lock();
        *output << out.str();
    }

private:
    template<std::size_t... I> void make_evaluators(std::index_sequence<I...>) {
        int dummy[] = {0, (evaluators->emplace_back(ensure_expr(std::get<I>(exprs).expr).get()), 0)...};
        (void)dummy;
    }

    template<std::size_t... I> void print_values(std::ostringstream& out, const IDouble* box, std::index_sequence<I...>) const {
        int dummy[] = {0, (out << '\t' << std::get<I>(exprs).name << ": " << (*evaluators)[I](box) << std::endl, 0)...};
        (void)dummy;
    }

    const ArgNameLookup* name_lookup;
    std::size_t num_args;
    std::ostream* output;
    std::tuple<OutputExprs...> exprs;
    std::shared_ptr<std::vector<sid_fe::HostEvaluator>> evaluators;
    std::shared_ptr<std::mutex> mtx = std::make_shared<std::mutex>();
};

template<typename... PrintExprs>
inline auto critical_printer(std::ostream& output, const ConstraintSystem& cs, PrintExprs&&... exprs) {
    return CriticalPrinter<false, std::decay_t<PrintExprs>...>{&cs, cs.num_args(), &output,
                                                              std::forward<PrintExprs>(exprs)...};
}

template<typename... PrintExprs>
inline auto locked_critical_printer(std::ostream& output, const ConstraintSystem& cs, PrintExprs&&... exprs) {
    return CriticalPrinter<true, std::decay_t<PrintExprs>...>{&cs, cs.num_args(), &output,
                                                             std::forward<PrintExprs>(exprs)...};
}

} // namespace ivarp

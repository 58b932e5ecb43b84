// Critical-cuboid printer (the reference's ivarp/critical_printer.hpp:27-110).
#pragma once

#include <mutex>
#include <ostream>
#include <sstream>
#include <string>
#include <tuple>
#include <utility>

#include "prover.hpp"

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

/// Prints every critical cuboid: one line per variable. The extra expressions are listed by name; their
/// interval values are not evaluated on the host (the proof path has no CPU evaluator).
template<bool Locking, typename... OutputExprs> class CriticalPrinter {
public:
    CriticalPrinter(const ArgNameLookup* lookup, std::size_t num_args, std::ostream* output, OutputExprs... exprs) :
        name_lookup(lookup), num_args(num_args), output(output), exprs(std::move(exprs)...) {}

    template<typename Context, typename ValueArray> void operator()(const Context&, const ValueArray& values) const {
        std::ostringstream out;
        out << "Critical:\n";
        for(std::size_t i = 0; i < num_args; ++i) {
            out << '\t' << name_lookup->arg_name(i) << ": " << values[i] << std::endl;
        }
        print_names(out, std::index_sequence_for<OutputExprs...>{});
        std::unique_lock<std::mutex> lock(*mtx, std::defer_lock);
        if(Locking) lock.lock();
        *output << out.str();
    }

private:
    template<std::size_t... I> void print_names(std::ostringstream& out, std::index_sequence<I...>) const {
        int dummy[] = {0, (out << '\t' << std::get<I>(exprs).name << ": (expression)" << std::endl, 0)...};
        (void)dummy;
    }

    const ArgNameLookup* name_lookup;
    std::size_t num_args;
    std::ostream* output;
    std::tuple<OutputExprs...> exprs;
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

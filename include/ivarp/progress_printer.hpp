// Progress printer (the reference's ivarp/progress_printer.hpp:37-98): prints queue size, cuboid
// count (critical count) and the first variables of one queued element.
#pragma once

#include <algorithm>
#include <cstdio>
#include <exception>
#include <ostream>
#include <sstream>
#include <string>
#include <unistd.h>

#include "run_prover.hpp"

namespace ivarp {

inline bool stdstream_is_tty(std::ostream& stream) {
    if(&stream == &std::cout) return isatty(fileno(stdout)) != 0;
    if(&stream == &std::cerr || &stream == &std::clog) return isatty(fileno(stderr)) != 0;
    return false;
}

class ProgressPrinter {
public:
    ProgressPrinter(std::ostream& output, std::size_t max_num_vars, const ConstraintSystem* arg_names) :
        output(&output), output_is_tty(stdstream_is_tty(output)),
        max_num_vars(std::min(max_num_vars, arg_names->num_args())), arg_names(arg_names) {}

    template<typename Context, typename EntryType>
    void observe_progress(const Context&, const EntryType& queue_head, const ProgressInfo& info) {
        std::ostringstream buffer;
        buffer << "Queue size: " << info.queue_size << ", cuboids: " << info.cuboid_count << "("
               << info.critical_count << ')';
        for(std::size_t i = 0; i < max_num_vars; ++i) {
            buffer << ", " << arg_names->arg_name(i) << ": " << queue_head.elements[i];
        }
        std::string str = buffer.str();
        if(str.size() > max_chars_printed) max_chars_printed = str.size();
        else if(output_is_tty) str.append(max_chars_printed - str.size(), ' ');
        if(output_is_tty) str.append(max_chars_printed, '\b'); else str += '\n';
        *output << str;
        if(output_is_tty) output->flush();
    }

    void observe_done() const {
        if(max_chars_printed > 0 && output_is_tty) {
            std::string buf(max_chars_printed, ' ');
            buf.append(max_chars_printed, '\b');
            *output << buf << std::flush;
        }
    }

    void observe_error(std::exception_ptr, std::size_t error_thread_id) {
        observe_done();
        *output << "Proof aborting with error thrown by prover thread #" << error_thread_id << std::endl;
    }

private:
    std::ostream* output;
    bool output_is_tty;
    std::size_t max_num_vars;
    std::size_t max_chars_printed{0};
    const ConstraintSystem* arg_names;
};

} // namespace ivarp

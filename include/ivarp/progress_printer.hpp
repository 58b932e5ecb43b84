// Progress output for proofs run through ivarp::run_prover.
//
// The lemma programs construct `ivarp::ProgressPrinter printer(std::cout, 3, &system)` and pass it to
// run_prover (src/proof_auxiliaries.hpp:46 in the reference); the engine calls the observer between steps
// with the queue size, the cuboid and critical counts and one queued element. The text written per update
// is the reference's (ivarp/include/ivarp/progress_printer.hpp:47-61): "Queue size: Q, cuboids: C(K)"
// followed by ", name: [lo, hi]" for the first variables. On a terminal the updates redraw one line in
// place; any other stream receives one line per update.
#pragma once

#include <cstdio>
#include <exception>
#include <iostream>
#include <ostream>
#include <sstream>
#include <string>
#include <unistd.h>

#include "run_prover.hpp"

namespace ivarp {

/// Whether a standard stream writes to a terminal (other streams never do).
inline bool stdstream_is_tty(std::ostream& stream) {
    int fd = -1;
    if(&stream == &std::cout) fd = fileno(stdout);
    else if(&stream == &std::cerr || &stream == &std::clog) fd = fileno(stderr);
    return fd >= 0 && isatty(fd) != 0;
}

namespace progress_detail {

/// The text of one progress update.
template<typename Names, typename Entry>
std::string progress_text(const ProgressInfo& info, const Entry& head, std::size_t shown_vars, const Names& names) {
    std::ostringstream s;
    s << "Queue size: " << info.queue_size << ", cuboids: " << info.cuboid_count << '(' << info.critical_count << ')';
    for(std::size_t v = 0; v < shown_vars; ++v) s << ", " << names.arg_name(v) << ": " << head.elements[v];
    return s.str();
}

/// A status line. On a terminal each text replaces the previous one: it is padded with blanks to the width
/// of the widest text shown so far and followed by as many backspaces, so the cursor stays at the start of
/// the line; erase() blanks the line the same way. On other streams each text is one line and erase() writes
/// nothing.
class StatusLine {
public:
    explicit StatusLine(std::ostream& os) : os_(&os), tty_(stdstream_is_tty(os)) {}

    void show(std::string text) {
        if(!tty_) {
            *os_ << text << '\n';
            return;
        }
        if(text.size() < width_) text.resize(width_, ' ');
        width_ = text.size();
        text.append(width_, '\b');
        *os_ << text << std::flush;
    }

    void erase() const {
        if(!tty_ || width_ == 0) return;
        *os_ << std::string(width_, ' ') << std::string(width_, '\b') << std::flush;
    }

    std::ostream& stream() const { return *os_; }

private:
    std::ostream* os_;
    bool tty_;
    std::size_t width_ = 0;
};

} // namespace progress_detail

/// Progress observer printing to a stream (the reference's ProgressPrinter interface: observe_progress,
/// observe_done, observe_error).
class ProgressPrinter {
public:
    ProgressPrinter(std::ostream& output, std::size_t max_num_vars, const ConstraintSystem* arg_names) :
        line_(output), names_(arg_names),
        shown_vars_(max_num_vars < arg_names->num_args() ? max_num_vars : arg_names->num_args()) {}

    template<typename Context, typename EntryType>
    void observe_progress(const Context&, const EntryType& queue_head, const ProgressInfo& info) {
        line_.show(progress_detail::progress_text(info, queue_head, shown_vars_, *names_));
    }

    void observe_done() const { line_.erase(); }

    void observe_error(std::exception_ptr, std::size_t error_thread_id) {
        line_.erase();
        line_.stream() << "Proof aborting with error thrown by prover thread #" << error_thread_id << std::endl;
    }

private:
    progress_detail::StatusLine line_;
    const ConstraintSystem* names_;
    std::size_t shown_vars_;
};

} // namespace ivarp

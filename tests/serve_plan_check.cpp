// Test driver of the request-scheduling planner (squares-in-disk_gb300/csrc/serve_plan.hpp) for
// tests/test_serve_plan.py. Reads one command per line from stdin and prints the answer:
//   admit <used> <budget> <running> <free_slots> <bytes...>   ->  number admitted
//   fill <cap> <slot> <qsize> [<slot> <qsize> ...]            ->  "slot begin count dst" per take, ";"-separated
//   need <qsize> <taken> <fanout>                             ->  queue_need
//   grow <cap> <need>                                         ->  grow_capacity
//   bytes <nargs> <queue_cap> <crit_cap>                      ->  request_bytes
#include <cstdio>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "serve_plan.hpp"

using namespace sid::plan;

int main() {
    std::string line;
    while(std::getline(std::cin, line)) {
        std::istringstream in(line);
        std::string cmd;
        in >> cmd;
        if(cmd == "admit") {
            unsigned long long used, budget, running, free_slots, b;
            in >> used >> budget >> running >> free_slots;
            std::vector<std::uint64_t> bytes;
            while(in >> b) bytes.push_back(b);
            std::cout << admit_count(bytes, used, budget, running, free_slots) << "\n";
        } else if(cmd == "fill") {
            unsigned long long cap, q;
            int slot;
            in >> cap;
            std::vector<std::pair<int, std::uint64_t>> active;
            while(in >> slot >> q) active.emplace_back(slot, q);
            bool first = true;
            for(const Take& t : fill_step(active, cap)) {
                std::cout << (first ? "" : ";") << t.slot << " " << t.begin << " " << t.count << " " << t.dst;
                first = false;
            }
            std::cout << "\n";
        } else if(cmd == "need") {
            unsigned long long q, t, f;
            in >> q >> t >> f;
            std::cout << queue_need(q, t, f) << "\n";
        } else if(cmd == "grow") {
            unsigned long long c, n;
            in >> c >> n;
            std::cout << grow_capacity(c, n) << "\n";
        } else if(cmd == "bytes") {
            int nargs;
            unsigned long long qc, cc;
            in >> nargs >> qc >> cc;
            std::cout << request_bytes(nargs, qc, cc) << "\n";
        }
    }
    return 0;
}

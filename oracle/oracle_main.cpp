// CPU ORACLE -- test infrastructure only: command line front end.
//   oracle_cli prove <file.sidir> [generations] [threads] [fp32]   (fp32: the precision form)
#include "oracle.hpp"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>

int main(int argc, char** argv) {
    if(argc < 3) {
        std::fprintf(stderr, "usage: %s prove <lemma.sidir> [generations] [threads] [fp32]\n", argv[0]);
        return 2;
    }
    std::ifstream in(argv[2]);
    std::stringstream ss;
    ss << in.rdbuf();
    sido::ProveOptions o;
    if(argc > 3) o.generations = unsigned(std::atoi(argv[3]));
    if(argc > 4) o.threads = std::atoi(argv[4]);
    if(argc > 5) o.fp32_first = std::string(argv[5]) == "fp32";
    try {
        sido::ProveResult r = sido::prove(ss.str(), o);
        std::printf("cuboids %llu leaves %llu criticals %llu repeated %llu seconds %.6f fp32_refuted %llu escalated %llu\n",
                    (unsigned long long)r.counts.cuboids, (unsigned long long)r.counts.leaves,
                    (unsigned long long)r.counts.criticals, (unsigned long long)r.counts.repeated, r.seconds,
                    (unsigned long long)r.counts.fp32_refuted, (unsigned long long)r.counts.escalated);
    } catch(const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}

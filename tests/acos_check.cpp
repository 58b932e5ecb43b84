// Test driver of the directed arc cosine in squares-in-disk_gb300/csrc/acos.cuh, for tests/test_acos.py.
// Built twice from this one file: for the host with g++, and for the GPU with nvcc (-x cu), where the
// same routine runs inside a kernel, one argument per thread.
//
// Reads lines "<d|f> <hex bits of a double>" from stdin and prints, per line, the hex bit patterns of
// acos rounded down and up (double for 'd', float for 'f'), whether the two-limb and the four-limb
// evaluations decide the rounding on their own (1/0; -1 outside [-1, 1)), and the downward rounding
// taken from the four-limb evaluation alone (0 where it is undecided or x is outside [-1, 1)).
#include <cinttypes>
#include <cstdio>
#include <vector>

#include "acos.cuh"

using namespace sid::acos_cr;

struct Case {
    double x;
    int is_float;
};

struct Out {
    std::uint64_t rd, ru, rd4;
    int dec2, dec4;
};

SID_ACOS_HD inline Out check_one(Case c) {
    int digits = c.is_float ? 24 : 53;
    Out o;
    o.dec2 = -1;
    o.dec4 = -1;
    o.rd4 = 0;
    // the product's float path converts float arguments to double bits with integer operations
    const std::uint64_t xb = c.is_float ? f32_to_f64_bits(float_bits(float(c.x))) : bits_of(c.x);
    if(c.x >= -1.0 && c.x < 1.0) {
        std::uint64_t m, mh;
        int l, lh;
        o.dec2 = acos_floor<2>(xb, digits, m, l, mh, lh) ? 1 : 0;
        o.dec4 = acos_floor<4>(xb, digits, m, l, mh, lh) ? 1 : 0;
        if(o.dec4) {
            int bias = digits == 53 ? 1023 : 127;
            o.rd4 = (static_cast<std::uint64_t>(l - (64 * 4 - 3) + bias) << (digits - 1)) |
                    (m & ((std::uint64_t(1) << (digits - 1)) - 1));
        }
    }
    if(c.is_float) {
        o.rd = float_bits(acos_rd(float(c.x)));
        o.ru = float_bits(acos_ru(float(c.x)));
    } else {
        o.rd = bits_of(acos_rd(c.x));
        o.ru = bits_of(acos_ru(c.x));
    }
    return o;
}

#if defined(__CUDACC__)
__global__ void k_check(const Case* in, Out* out, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i < n) out[i] = check_one(in[i]);
}

static bool run_all(const std::vector<Case>& in, std::vector<Out>& out) {
    int n = static_cast<int>(in.size());
    Case* din = nullptr;
    Out* dout = nullptr;
    if(cudaMalloc(&din, sizeof(Case) * n) != cudaSuccess) return false;
    if(cudaMalloc(&dout, sizeof(Out) * n) != cudaSuccess) return false;
    cudaMemcpy(din, in.data(), sizeof(Case) * n, cudaMemcpyHostToDevice);
    k_check<<<(n + 127) / 128, 128>>>(din, dout, n);
    cudaError_t e = cudaMemcpy(out.data(), dout, sizeof(Out) * n, cudaMemcpyDeviceToHost);
    cudaFree(din);
    cudaFree(dout);
    if(e != cudaSuccess) std::fprintf(stderr, "CUDA error: %s\n", cudaGetErrorString(e));
    return e == cudaSuccess;
}
#else
static bool run_all(const std::vector<Case>& in, std::vector<Out>& out) {
    for(std::size_t i = 0; i < in.size(); ++i) out[i] = check_one(in[i]);
    return true;
}
#endif

int main() {
    std::vector<Case> in;
    char kind;
    unsigned long long bits;
    while(std::scanf(" %c %llx", &kind, &bits) == 2) in.push_back({double_of(bits), kind == 'f' ? 1 : 0});
    if(in.empty()) return 0;
    std::vector<Out> out(in.size());
    if(!run_all(in, out)) return 1;
    for(const Out& o : out) {
        std::printf("%" PRIx64 " %" PRIx64 " %d %d %" PRIx64 "\n", o.rd, o.ru, o.dec2, o.dec4, o.rd4);
    }
    return 0;
}

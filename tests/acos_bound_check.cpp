// Test driver of acos_bound_f32 (squares-in-disk_gb300/csrc/acos.cuh), the float pass's arc cosine bound,
// for tests/test_acos.py and tests/test_gpu_acos.py. Built for the host with g++ (which runs the bound in the
// FE_DOWNWARD rounding mode it requires) and for the GPU with nvcc (-x cu; directed-rounding intrinsics).
//
//   acos_bound_check            reads float bit patterns (hex) from stdin, prints per line the bits of the
//                               lower and upper bound and of the correctly rounded acos rounded down and up
//   acos_bound_check coef       the float bounds of the series coefficients (hex bits, lower and upper)
//   acos_bound_check sweep S    every S-th float of [-1, 1] (all 2,130,706,434 of them for S = 1): prints
//                               "checked violations first_bad max_width_ulps sum_width_ulps", where a
//                               violation is lower > acos rounded down or upper < acos rounded up (acos(x) is
//                               transcendental for x != 1, so these are exactly the unsound bounds)
#include <cfenv>
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "acos.cuh"

using namespace sid::acos_cr;

namespace {

constexpr std::uint64_t kPositive = 0x3f800001ull;   // bit patterns +0 .. 1.0
constexpr std::uint64_t kSweepTotal = 2 * kPositive;

SID_ACOS_HD inline std::uint32_t sweep_bits(std::uint64_t i) {
    return i < kPositive ? std::uint32_t(i) : (0x80000000u | std::uint32_t(i - kPositive));
}

// order-preserving integer of a float: ulps between two floats are differences of these
SID_ACOS_HD inline std::int64_t ordered(float f) {
    const std::uint32_t b = float_bits(f);
    return (b & 0x80000000u) ? -std::int64_t(b & 0x7fffffffu) : std::int64_t(b);
}

struct Row {
    std::uint32_t lo, hi, rd, ru;
};

struct Summary {
    unsigned long long checked, violations, first_bad, max_width, sum_width;
};

SID_ACOS_HD inline void check_one(std::uint32_t b, Row& r) {
    const float x = float_of(b);
    r.rd = float_bits(acos_rd(x));
    r.ru = float_bits(acos_ru(x));
#if !defined(__CUDA_ARCH__)
    std::fesetround(FE_DOWNWARD);
#endif
    r.lo = float_bits(acos_bound_f32(x, false));
    r.hi = float_bits(acos_bound_f32(x, true));
#if !defined(__CUDA_ARCH__)
    std::fesetround(FE_TONEAREST);
#endif
}

SID_ACOS_HD inline bool violates(const Row& r) {
    return !(float_of(r.lo) <= float_of(r.rd)) || !(float_of(r.hi) >= float_of(r.ru));
}

#if defined(__CUDACC__)
__global__ void k_rows(const std::uint32_t* in, Row* out, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i < n) check_one(in[i], out[i]);
}

// indices k0 <= k < k1 of the sweep (float index k * stride)
__global__ void k_sweep(std::uint64_t stride, std::uint64_t k0, std::uint64_t k1, Summary* s) {
    unsigned long long viol = 0, maxw = 0, sumw = 0, cnt = 0, first = ~0ull;
    const std::uint64_t step = std::uint64_t(gridDim.x) * blockDim.x;
    for(std::uint64_t k = k0 + std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < k1; k += step) {
        const std::uint64_t i = k * stride;
        Row r;
        check_one(sweep_bits(i), r);
        ++cnt;
        if(violates(r)) {
            ++viol;
            if(i < first) first = i;
        }
        const unsigned long long w = (unsigned long long)(ordered(float_of(r.hi)) - ordered(float_of(r.lo)));
        sumw += w;
        if(w > maxw) maxw = w;
    }
    atomicAdd(&s->checked, cnt);
    atomicAdd(&s->violations, viol);
    atomicMin(&s->first_bad, first);
    atomicMax(&s->max_width, maxw);
    atomicAdd(&s->sum_width, sumw);
}

bool run_rows(const std::vector<std::uint32_t>& in, std::vector<Row>& out) {
    const int n = int(in.size());
    std::uint32_t* din = nullptr;
    Row* dout = nullptr;
    if(cudaMalloc(&din, sizeof(std::uint32_t) * n) != cudaSuccess) return false;
    if(cudaMalloc(&dout, sizeof(Row) * n) != cudaSuccess) return false;
    cudaMemcpy(din, in.data(), sizeof(std::uint32_t) * n, cudaMemcpyHostToDevice);
    k_rows<<<(n + 127) / 128, 128>>>(din, dout, n);
    const cudaError_t e = cudaMemcpy(out.data(), dout, sizeof(Row) * n, cudaMemcpyDeviceToHost);
    cudaFree(din);
    cudaFree(dout);
    if(e != cudaSuccess) std::fprintf(stderr, "CUDA error: %s\n", cudaGetErrorString(e));
    return e == cudaSuccess;
}

bool run_sweep(std::uint64_t stride, Summary& s) {
    Summary* d = nullptr;
    if(cudaMalloc(&d, sizeof(Summary)) != cudaSuccess) return false;
    Summary init{0, 0, ~0ull, 0, 0};
    cudaMemcpy(d, &init, sizeof(Summary), cudaMemcpyHostToDevice);
    // launches of at most 2^26 floats each, so that no single kernel runs for long
    const std::uint64_t count = (kSweepTotal + stride - 1) / stride, per = std::uint64_t(1) << 26;
    cudaError_t e = cudaSuccess;
    for(std::uint64_t k0 = 0; k0 < count && e == cudaSuccess; k0 += per) {
        k_sweep<<<152 * 16, 128>>>(stride, k0, k0 + per < count ? k0 + per : count, d);
        e = cudaDeviceSynchronize();
    }
    if(e == cudaSuccess) e = cudaMemcpy(&s, d, sizeof(Summary), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if(e != cudaSuccess) std::fprintf(stderr, "CUDA error: %s\n", cudaGetErrorString(e));
    return e == cudaSuccess;
}
#else
bool run_rows(const std::vector<std::uint32_t>& in, std::vector<Row>& out) {
    for(std::size_t i = 0; i < in.size(); ++i) check_one(in[i], out[i]);
    return true;
}

bool run_sweep(std::uint64_t stride, Summary& s) {
    s = Summary{0, 0, ~0ull, 0, 0};
    for(std::uint64_t i = 0; i < kSweepTotal; i += stride) {
        Row r;
        check_one(sweep_bits(i), r);
        ++s.checked;
        if(violates(r)) {
            ++s.violations;
            if(i < s.first_bad) s.first_bad = i;
        }
        const unsigned long long w = (unsigned long long)(ordered(float_of(r.hi)) - ordered(float_of(r.lo)));
        s.sum_width += w;
        if(w > s.max_width) s.max_width = w;
    }
    return true;
}
#endif

} // namespace

int main(int argc, char** argv) {
    if(argc >= 2 && std::strcmp(argv[1], "coef") == 0) {   // the series coefficient bounds, lower then upper
        for(int k = 0; k < 11; ++k) std::printf("%08x %08x\n", float_bits(asin_coef(k, false)), float_bits(asin_coef(k, true)));
        return 0;
    }
    if(argc >= 3 && std::strcmp(argv[1], "sweep") == 0) {
        const std::uint64_t stride = std::strtoull(argv[2], nullptr, 10);
        if(stride == 0) return 2;
        Summary s;
        if(!run_sweep(stride, s)) return 1;
        std::printf("%llu %llu %llu %llu %llu\n", s.checked, s.violations, s.first_bad, s.max_width, s.sum_width);
        return 0;
    }
    std::vector<std::uint32_t> in;
    unsigned int bits;
    while(std::scanf(" %x", &bits) == 1) in.push_back(bits);
    if(in.empty()) return 0;
    std::vector<Row> out(in.size());
    if(!run_rows(in, out)) return 1;
    for(const Row& r : out) std::printf("%08x %08x %08x %08x\n", r.lo, r.hi, r.rd, r.ru);
    return 0;
}

// TEST INFRASTRUCTURE: the continuation network of the GPU least-squares Monte Carlo on
// the CPU -- its loss and parameter gradients on a batch, for gradient checks of the
// tensor-core training kernels.
//
// The network is f(x) = w3 . relu(W2 relu(W1 x + b1) + b2) + b3 with 3 inputs and two
// hidden layers of 64 units; parameters are packed as W1[64][3], b1[64], W2[64][64]
// (row = output unit), b2[64], w3[64], b3.  The loss is mean((f(x) - y)^2) over the
// batch.  With `bf16` set, the operands the GPU hands to its tensor cores are rounded
// to bfloat16 (round to nearest even) exactly where the GPU rounds them: the first
// hidden layer's activations, W2, the second layer's pre-activation gradients (in dW2,
// db2 and dH1), the first layer's pre-activation gradients and the inputs (in dW1 and
// db1), and the second layer's activations and the output gradient (in dW3); the rest
// is evaluated in double.  With `bf16` clear the whole computation is in double.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

constexpr int H = 64;
constexpr int PW1 = 0, PB1 = 192, PW2 = 256, PB2 = 4352, PW3 = 4416, PB3 = 4480, NP = 4481;

double bf16(double value) {
    float f = float(value);
    uint32_t u;
    std::memcpy(&u, &f, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    u &= 0xFFFF0000u;
    std::memcpy(&f, &u, 4);
    return double(f);
}

}  // namespace

extern "C" double kor_mlp_gradients(const float* params, const float* samples, int count, int bf16_operands,
                                    double* grads) {
    auto round = [&](double v) { return bf16_operands ? bf16(v) : v; };
    for (int i = 0; i < NP; ++i) grads[i] = 0.0;
    std::vector<double> w2(H * H);
    for (int i = 0; i < H * H; ++i) w2[i] = round(params[PW2 + i]);
    double loss = 0.0;
    std::vector<double> h1(H), z2(H), dz2(H);
    for (int r = 0; r < count; ++r) {
        const float* x = samples + 4 * r;
        unsigned long long mask1 = 0;
        for (int j = 0; j < H; ++j) {
            // The GPU evaluates layer 1 in FP32 with fused multiply-adds, then rounds.
            float z = std::fmaf(params[PW1 + 3 * j], x[0],
                                std::fmaf(params[PW1 + 3 * j + 1], x[1], std::fmaf(params[PW1 + 3 * j + 2], x[2], params[PB1 + j])));
            double zd = bf16_operands ? double(z)
                                      : double(params[PW1 + 3 * j]) * x[0] + double(params[PW1 + 3 * j + 1]) * x[1] +
                                            double(params[PW1 + 3 * j + 2]) * x[2] + double(params[PB1 + j]);
            if (zd > 0.0) mask1 |= 1ull << j;
            h1[j] = round(zd > 0.0 ? zd : 0.0);
        }
        double out = params[PB3];
        for (int o = 0; o < H; ++o) {
            double z = 0.0;
            for (int i = 0; i < H; ++i) z += w2[o * H + i] * h1[i];
            z2[o] = z + params[PB2 + o];
            out += (z2[o] > 0.0 ? z2[o] : 0.0) * params[PW3 + o];
        }
        const double res = out - double(x[3]);
        loss += res * res;
        const double dout = 2.0 * res / double(count);
        grads[PB3] += dout;
        for (int o = 0; o < H; ++o) {
            const bool on = z2[o] > 0.0;
            grads[PW3 + o] += round(dout) * round(on ? z2[o] : 0.0);
            const double g = on ? dout * params[PW3 + o] : 0.0;
            dz2[o] = round(g);
            grads[PB2 + o] += dz2[o];
        }
        for (int o = 0; o < H; ++o)
            for (int i = 0; i < H; ++i) grads[PW2 + o * H + i] += dz2[o] * h1[i];
        for (int i = 0; i < H; ++i) {
            if (!((mask1 >> i) & 1ull)) continue;
            double dh = 0.0;
            for (int o = 0; o < H; ++o) dh += dz2[o] * w2[o * H + i];
            dh = round(dh);
            grads[PW1 + 3 * i] += dh * round(x[0]);
            grads[PW1 + 3 * i + 1] += dh * round(x[1]);
            grads[PW1 + 3 * i + 2] += dh * round(x[2]);
            grads[PB1 + i] += dh;
        }
    }
    return loss / double(count);
}

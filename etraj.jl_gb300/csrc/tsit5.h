// tsit5.h -- the Tsit5 tableau (Tsitouras 2011, the coefficients OrdinaryDiffEq
// uses) as compile-time FP64 constants, with the products the second-order
// (Nystrom) form of a step needs.  Row 6 of kA is the solution weights b
// (first same as last: stage 7 is the derivative at the new state); kBT is
// b - b_hat of the embedded fourth-order estimate.
#pragma once

namespace etraj {
namespace tsit5 {

constexpr double kC[7] = {0.0, 0.161, 0.327, 0.9, 0.9800255409045097, 1.0, 1.0};
constexpr double kA[7][7] = {
    {0, 0, 0, 0, 0, 0, 0},
    {0.161, 0, 0, 0, 0, 0, 0},
    {-0.008480655492356989, 0.335480655492357, 0, 0, 0, 0, 0},
    {2.897153057105493, -6.359448489975075, 4.3622954328695815, 0, 0, 0, 0},
    {5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525, 0, 0, 0},
    {5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383, 0, 0},
    {0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774, 0}};
constexpr double kBT[7] = {-0.00178001105222577714, -0.0008164344596567469, 0.007880878010261995,
                           -0.1447110071732629, 0.5823571654525552, -0.45808210592918697,
                           0.015151515151515152};

// (A A)[i][l]: the weight of stage derivative l in the position of stage i when
// positions advance as x + (sum_l A_il) dt p + dt^2 sum_l (A A)_il K_l (x' = p, p' = K)
constexpr double aa(int i, int l) {
    double s = 0.0;
    for (int j = 0; j < 7; ++j) s += kA[i][j] * kA[j][l];
    return s;
}
// (bt A)[l]: the same for the position rows of the error estimate
constexpr double bta(int l) {
    double s = 0.0;
    for (int i = 0; i < 7; ++i) s += kBT[i] * kA[i][l];
    return s;
}
// row sums of A and of A A
constexpr double rowsum_a(int i) {
    double s = 0.0;
    for (int l = 0; l < 7; ++l) s += kA[i][l];
    return s;
}
constexpr double rowsum_aa(int i) {
    double s = 0.0;
    for (int l = 0; l < 7; ++l) s += aa(i, l);
    return s;
}

}  // namespace tsit5
}  // namespace etraj

// pfa_model.h -- model data of the KKS Cr-Nb-Ni paraboloid model, shared by
// host and device code of libpfa_gb300.
//
// The numbers are the model data baked into the reference's generated
// thermo/parabola625.c (usnistgov/phasefield-precipitate-aging); they are
// arranged here as coefficient tables:
//   equilibrium compositions          thermo/parabola625.c:65-117
//   paraboloids g_gam, g_del, g_lav   thermo/parabola625.c:418-443
//   gamma chemical potential          thermo/parabola625.c:655-671
//   fictitious compositions           thermo/parabola625.c:245-297
//   diffusivities D_CrCr ... D_NbNb   thermo/parabola625.c:1860-1894
//   kT, RT, Vm, sigma                 thermo/parabola625.c:38-63,299-315
#pragma once

#ifdef __CUDACC__
#define PFA_HD __host__ __device__ __forceinline__
#else
#define PFA_HD inline
#endif

namespace pfa {

constexpr double kKT = 1.5782889043500002e-20;
constexpr double kRT = 9504.6840941999999;
constexpr double kVm = 1.0000000000000001e-5;
constexpr double kSigma = 0.13;
constexpr double kLatticeConst = 0.352e-9;  // src/parameters.h:26
constexpr double kOmega = 1.07e11;          // src/parameters.h:37
constexpr double kPi = 3.14159265358979323846;

// [phase: gam, del, lav][comp: Cr, Nb]
constexpr double kXe[3][2] = {
    {0.52421634830562147, 0.01299272922003303},
    {0.022966218927631978, 0.24984563695705883},
    {0.37392129441013022, 0.25826261799015571},
};

// g = A (XCR - xeCr)^2 + (B XCR - C)(XNB - xeNb) + E (XNB - xeNb)^2 ; columns A B C E
constexpr double kG[3][4] = {
    {2267132212.7620249, 15095482346.486225, 7913298631.5869827, 55193083240.685936},
    {21346492990.798885, 16906497386.287418, 388278320.27291465, 3085369132931.8848},
    {8866730284.8069954, 24191004361.532181, 9045531663.945219, 98294310279.883911},
};

// d g_gam / d x_k = a XCR + b XNB + c
constexpr double kDg[2][3] = {
    {4534264425.5240498, 15095482346.486225, -2573067053.9739881},
    {15095482346.486225, 110386166481.37187, -9347516202.3169327},
};

// d g_<phase> / d x_<comp> = a XCR + b XNB + c for every phase (gamma, delta,
// laves), and the constant curvatures d2 g_<phase> / d x_i d x_j
// (thermo/parabola625.c:655-706, 1305-1410)
constexpr double kDgPh[3][2][3] = {
    {{4534264425.5240498, 15095482346.486225, -2573067053.9739881},
     {15095482346.486225, 110386166481.37187, -9347516202.3169327}},
    {{42692985981.597771, 16906497386.287418, -5204511070.9175282},
     {16906497386.287418, 6170738265863.7695, -1542120310850.303}},
    {{17733460569.613991, 24191004361.532181, -12878550648.781645},
     {24191004361.532181, 196588620559.76782, -59817023476.78421}},
};
constexpr double kD2g[3][2][2] = {
    {{4534264425.5240498, 15095482346.486225}, {15095482346.486225, 110386166481.37187}},
    {{42692985981.597771, 16906497386.287418}, {16906497386.287418, 6170738265863.7695}},
    {{17733460569.613991, 24191004361.532181}, {24191004361.532181, 196588620559.76782}},
};

// shared denominator of the fictitious compositions over the monomials
// [pD^2, pD pG, pD pL, pG^2, pG pL, pL^2]
constexpr double kDen[6] = {0.001036042775998007, 0.12229015747171917, 0.041785936156220213,
                            1.0, 0.73028945399293654, 0.093983883345629876};

// numerators: scale * (XCR (l . [pD pG pL]) + XNB (m . [pD pG pL]) + q . monomials)
struct FictRow {
  double scale, l[3], m[3], q[6];
};
constexpr FictRow kFict[3][2] = {
    {{1.0, {0.016938286205500769, 1.0, 0.54889980006097594},
      {-0.3468746660495467, 0.0, -0.10246420218061991},
      {0.086819224054883945, 0.036767802923980249, 0.11815012520929236, 0.0,
       -0.27750258277182049, -0.12951476250779617}},
     {-1.0, {0.0021576593653206376, 0.0, 0.054466450838266962},
      {-0.10535187126621841, -1.0, -0.18138965393196074},
      {0.026258691080522339, 0.24849448207756414, 0.06992726713680375, 0.0,
       0.22257870755542869, 0.025258893954068839}}},
    {{0.3468746660495467, {0.0029867928603642137, 0.30371739875396442, 0.11224396861282376},
      {0.0, 1.0, 0.15026949298026254},
      {0.0, -0.25028989589710454, -0.038472217853981416, -0.10599737173866837,
       -0.38426983287411109, -0.074556825343604527}},
     {0.24849448207756414, {0.0, 0.0086829266681549659, 0.0010534256500958396},
      {0.0041692787998190662, 0.068163631095090937, 0.011474488301439056},
      {0.0, 0.10567112340275649, 0.038045328588644858, 1.0, 0.71270814650507497,
       0.091137578230976013}}},
    {{0.27750258277182055, {0.010275028791049912, 0.65365032685519298, 0.33867750853659306},
      {-0.18783493715380425, 0.36923693162478488, 0.0},
      {0.04808977843373196, 0.054570103782716275, 0.093195074562756067, 1.0,
       0.46671552103819908, 0.0}},
     {-0.54889980006097605, {0.00047690026722310247, -0.099228403494073802, 0.0},
      {-0.070932051941581864, -1.0, -0.1712222947342838},
      {0.017223643043877624, 0.19525744879034301, 0.041259234012827196, -0.40549970601319757,
       -0.046017313089315913, 0.0}}},
};

// Diffusivity data: mobility prefactors and exponents, and the curvature
// weights (the additive copies carry their own last digits in the source).
constexpr double kMobPreNb = 1.4170990277916469e-20;
constexpr double kMobPreCr = 3.5027570743586952e-21;
constexpr double kMobPreNi = 1.8295676400933012e-21;
constexpr double kHCrCr = 45342.644255240499;
constexpr double kHCrNb = 150954.82346486227;
constexpr double kHNbNb = 1103861.6648137188;
constexpr double kHCrNbAddA = 150954.82346486227;
constexpr double kHCrNbAddB = 150954.82346486225;
constexpr double kHNbNbAdd = 1103861.664813719;
constexpr double kHCrCrAdd = 45342.644255240499;

}  // namespace pfa

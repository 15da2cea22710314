// rift_device.cuh -- per-cell and per-face arithmetic of the GB300 step.
//
// The state is FP32 depth h (not surface elevation w), so the wet threshold
// epsilon (1.19e-7 m, grid.cu:29) is resolved at any bed elevation.  Every
// bed elevation enters through FP32 differences precomputed in FP64:
//   eW, eE : west / east face elevation minus the cell's reference elevation
//   eS, eN : south / north face elevation minus the same
// so w_{i+1} - w_i = (eE_i - eW_{i+1}) + (h_{i+1} - h_i) and the face depth
// w_face - B_face = h +- slope - e_face, with no large absolute elevation ever
// rounded to FP32.
#pragma once
#include <cstdint>

namespace rift {

constexpr float kG = 9.80665f;         // grid.cu:28
constexpr float kEps = 1.19209e-07f;   // grid.cu:29
constexpr float kTheta = 1.3f;         // grid.cu:30

// Effective limiter of the reference (grid.cu:62-80).  Its signf reads the
// low word of a double and is never negative, so minmod(a,b,c) evaluates to
// +min(|a|,|b|,|c|) (times a factor within 1.5e-6 of 1) and the slope is
//   0.5 * min(theta|d+|, 0.5|d+ + d-|, theta|d-|)  >= 0.
// It is zero whenever one argument is zero, which min() already gives.
// The outer factor 0.5 is folded into the three terms (0.65 = 1.3 / 2 and
// 0.25 exactly, so each product is the same float as half the unfolded one).
__device__ __forceinline__ float slope(float dp, float dm) {
    constexpr float kHalfTheta = 0.5f * kTheta;
    float a = kHalfTheta * fabsf(dp);
    float b = 0.25f * fabsf(dp + dm);
    float c = kHalfTheta * fabsf(dm);
    return fminf(fminf(a, b), c);
}

// Reconstructed face values of one cell in one direction (Construct,
// grid.cu:91-116), in depth form.  P = the face toward +x (+y), M = toward -x.
struct Rec {
    float hP, uP, vP;  // depth, hu, hv at the + face
    float hM, uM, vM;  // at the - face
};

// h0/u0/v0: the cell; hp../hm..: its + and - neighbours in this direction;
// eM/eP: the cell's - and + face elevation offsets; dP, dM: reference
// elevation steps to the + and - neighbour.
__device__ __forceinline__ Rec construct(float h0, float u0, float v0, float hp, float up, float vp,
                                         float hm, float um, float vm, float eM, float eP,
                                         float dP, float dM) {
    float sw = slope(dP + (hp - h0), dM + (h0 - hm));
    float su = slope(up - u0, u0 - um);
    float sv = slope(vp - v0, v0 - vm);
    Rec r;
    float hP = (h0 + sw) - eP;
    float hM = (h0 - sw) - eM;
    // wet/dry correction against the face elevations; wBar = 2w, so the
    // corrected depth on the other face is 2h - eP - eM.
    float hBar = (h0 + h0) - (eP + eM);
    if (hP < 0.f) {
        hP = 0.f;
        hM = hBar;
    }
    if (hM < 0.f) {
        hP = hBar;
        hM = 0.f;
    }
    r.hP = hP;
    r.hM = hM;
    r.uP = u0 + su;
    r.uM = u0 - su;
    r.vP = v0 + sv;
    r.vM = v0 - sv;
    return r;
}

// Depth-only part of the reconstruction (speed pass): depth and the normal
// momentum at the two faces.
struct RecN {
    float hP, qP, hM, qM;
};

__device__ __forceinline__ RecN constructN(float h0, float q0, float hp, float qp, float hm,
                                           float qm, float eM, float eP, float dP, float dM) {
    float sw = slope(dP + (hp - h0), dM + (h0 - hm));
    float sq = slope(qp - q0, q0 - qm);
    float hP = (h0 + sw) - eP;
    float hM = (h0 - sw) - eM;
    float hBar = (h0 + h0) - (eP + eM);
    if (hP < 0.f) {
        hP = 0.f;
        hM = hBar;
    }
    if (hM < 0.f) {
        hP = hBar;
        hM = 0.f;
    }
    RecN r;
    r.hP = hP;
    r.hM = hM;
    r.qP = q0 + sq;
    r.qM = q0 - sq;
    return r;
}

// Desingularised velocity factor 2h / (h^2 + max(h^2, kappa)) (grid.cu:82-84).
__device__ __forceinline__ float velFactor(float h, float kappa) {
    float h2 = h * h;
    return (2.f * h) / (h2 + fmaxf(h2, kappa));
}

// Local speed at a face (the mx / my of getHX / getHY, grid.cu:118-214),
// from the upstream cell's + face (L) and the downstream cell's - face (R);
// qn is the momentum normal to the face.
__device__ __forceinline__ float faceSpeed(float hL, float qL, float hR, float qR, float kappa) {
    float uL = qL * velFactor(hL, kappa);
    float uR = qR * velFactor(hR, kappa);
    float cL = sqrtf(kG * hL), cR = sqrtf(kG * hR);
    float ap = fmaxf(fmaxf(uL + cL, uR + cR), 0.f);
    float am = fminf(fminf(uL - cL, uR - cR), 0.f);
    return fmaxf(ap, -am);
}

// Central-upwind numerical flux through one face (getHX for DIR 0, getHY for
// DIR 1; grid.cu:118-214, computeH grid.cu:86-89).  f[0] mass, f[1] x
// momentum, f[2] y momentum.  Returns the local speed max(a+, -a-).
template <int DIR>
__device__ __forceinline__ float faceFlux(float hL, float huL, float hvL, float hR, float huR,
                                          float hvR, float kappa, float f[3]) {
    float rL = velFactor(hL, kappa), rR = velFactor(hR, kappa);
    float uL = huL * rL, vL = hvL * rL, uR = huR * rR, vR = hvR * rR;
    // momenta recomputed from the desingularised velocities
    float quL = hL * uL, qvL = hL * vL, quR = hR * uR, qvR = hR * vR;
    float cL = sqrtf(kG * hL), cR = sqrtf(kG * hR);
    float nL = DIR == 0 ? uL : vL;
    float nR = DIR == 0 ? uR : vR;
    float ap = fmaxf(fmaxf(nL + cL, nR + cR), 0.f);
    float am = fminf(fminf(nL - cL, nR - cR), 0.f);
    float pL = 0.5f * kG * hL * hL, pR = 0.5f * kG * hR * hR;
    float FL0, FL1, FL2, FR0, FR1, FR2;
    if (DIR == 0) {
        FL0 = quL;
        FL1 = quL * uL + pL;
        FL2 = quL * vL;
        FR0 = quR;
        FR1 = quR * uR + pR;
        FR2 = quR * vR;
    } else {
        FL0 = qvL;
        FL1 = qvL * uL;
        FL2 = qvL * vL + pL;
        FR0 = qvR;
        FR1 = qvR * uR;
        FR2 = qvR * vR + pR;
    }
    if (!(hL > 0.f)) FL0 = FL1 = FL2 = 0.f;
    if (!(hR > 0.f)) FR0 = FR1 = FR2 = 0.f;
    float d = ap - am;
    if (d > 0.f) {
        float r = 1.f / d;
        float k = ap * am * r;
        f[0] = (ap * FL0 - am * FR0) * r + k * (hR - hL);
        f[1] = (ap * FL1 - am * FR1) * r + k * (quR - quL);
        f[2] = (ap * FL2 - am * FR2) * r + k * (qvR - qvL);
    } else {
        f[0] = f[1] = f[2] = 0.f;
    }
    return fmaxf(ap, -am);
}

// Green-Ampt infiltration rate (grid.cu:791-805), clamped to [0, h/dt].
// The quadratic root is taken in the cancellation-free form when p1 < 0.
__device__ __forceinline__ float greenAmpt(float K, float F, float psiDtheta, float dt, float hC) {
    float p1 = K * dt - 2.f * F;
    float p2 = K * (F + psiDtheta);
    float s = sqrtf(p1 * p1 + 8.f * p2 * dt);
    float f = (p1 >= 0.f) ? (p1 + s) / (2.f * dt) : (4.f * p2) / (s - p1);
    float cap = hC / dt;
    f = (f > cap) ? cap : f;
    f = (f > 0.f) ? f : 0.f;
    return f;
}

// Semi-implicit Manning coefficient G (grid.cu:754-760).
__device__ __forceinline__ float manningG(float n, float hu, float hv, float hC, float kappa) {
    float h2 = hC * hC;
    float den = h2 + fmaxf(h2, kappa);
    return -4.f * kG * n * n * sqrtf(hu * hu + hv * hv) * powf(hC, 5.f / 3.f) / (den * den);
}

// Critical-depth ghost value (ApplyBoundariesX_k / Y_k, grid.cu:1325-1406):
// min((q^2/g)^(1/3), h_interior).
__device__ __forceinline__ float criticalDepth(float q, float h) {
    return fminf(cbrtf(q * q / kG), h);
}

}  // namespace rift

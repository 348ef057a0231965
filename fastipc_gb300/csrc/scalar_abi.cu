// Host-side scalar functions with exactly the signatures of the reference's native library
// a.so (common/math/wrapper/wrapper.cpp:11-330), so that the reference's own ctypes glue
// (common/math/external_func.py:4, common/math/math_tools.py:78-181, common/math/ipc.py:382-411)
// can load libfastipc.so in its place.  Every input is a double by value, every output a double*
// slot; no return codes, no allocation and no global state, so the calls are reentrant like the
// reference's.  Each function runs this library's own math for one problem on the calling CPU
// thread: the same header code the GPU kernels use, compiled for the host here.
//
//   svd_2, svd_3                        wrapper.cpp:12-40   (svd2_givens below, nh.cuh svd3)
//   project_pd_{2,3,4,6,9,12}           wrapper.cpp:42-88   (eig.cuh Householder + QL projection)
//   solve_{2,3,4,6,9}                   wrapper.cpp:90-198  (pivoted LDL^T below)
//   get_smallest_positive_real_{quad,cubic}_root   wrapper.cpp:200-252 (ccd.cuh)
//   point_triangle_ccd, edge_edge_ccd   wrapper.cpp:254-328 (ccd.cuh EVCTCD with the step clamp)
//
// The GPU path never calls these: its kernels work on whole arrays (include/fastipc.h).
#include <math.h>
#include <string.h>

#include "../../include/fastipc_aso.h"
#include "ccd.cuh"
#include "ldlt.cuh"
#include "eig.cuh"
#include "fc2d.cuh"
#include "nh.cuh"

namespace {

using namespace fipc;

// n x n row-major symmetric `in` -> its PSD projection in `out` (the makePD rule of
// common/math/wrapper/UTILS.h:8-25: unchanged when the smallest eigenvalue is >= 0, otherwise
// every negative eigenvalue clamped to zero)
void project_pd_n(int n, const double* in, double* const* out) {
    double Q[PD_LD * PD_LD], lam[PD_LD];
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) Q[i * PD_LD + j] = in[i * n + j];
    sym_eig_ld<PD_LD>(n, Q, lam);
    if (lam[0] >= 0.0) {
        for (int i = 0; i < n * n; ++i) *out[i] = in[i];
        return;
    }
    // rebuilt from the non-negative part of the spectrum, as makePD rebuilds it: a matrix with
    // no positive eigenvalue comes back exactly zero
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            double s = 0.0;
            for (int k = 0; k < n; ++k)
                if (lam[k] > 0.0) s += lam[k] * Q[i * PD_LD + k] * Q[j * PD_LD + k];
            *out[i * n + j] = s;
        }
}

// 2x2 SVD in the convention of the reference's svd_2 (JGSL, wrapper.cpp:12-25): F = R S with R
// the rotation closest to F; S symmetric, diagonalised by one Jacobi rotation whose cosine is
// positive; singular values ordered s0 >= s1 (s1 may be negative), the rotation turned a
// quarter when they swap; U = R V.  Rotations are stored as (c, s) and filled as [[c, s], [-s, c]].
void svd2_givens(const double* F, double* U, double* sig, double* V) {
    double rc = 1.0, rs = 0.0;
    const double px = F[0] + F[3], py = F[2] - F[1];
    const double den = sqrt(px * px + py * py);
    if (den != 0.0) {
        rc = px / den;
        rs = -py / den;
    }
    // S = R^T F (row rotation of F)
    const double s00 = rc * F[0] - rs * F[2], s01 = rc * F[1] - rs * F[3];
    const double s11 = rs * F[1] + rc * F[3];
    double c = 1.0, sn = 0.0;
    const double x = s00, y = s01, z = s11, y2 = y * y;
    if (y2 == 0.0) {
        sig[0] = x;
        sig[1] = z;
    } else {
        const double tau = 0.5 * (x - z), w = sqrt(tau * tau + y2);
        const double t = tau > 0 ? y / (tau + w) : y / (tau - w);
        c = 1.0 / sqrt(t * t + 1.0);
        sn = -t * c;
        const double c2 = c * c, csy = 2 * c * sn * y, s2 = sn * sn;
        sig[0] = c2 * x - csy + s2 * z;
        sig[1] = s2 * x + csy + c2 * z;
    }
    double vc = c, vs = sn;
    if (sig[0] < sig[1]) {
        const double tmp = sig[0];
        sig[0] = sig[1];
        sig[1] = tmp;
        vc = -sn;
        vs = c;
    }
    const double uc = rc * vc - rs * vs, us = rs * vc + rc * vs;
    U[0] = uc, U[1] = us, U[2] = -us, U[3] = uc;
    V[0] = vc, V[1] = vs, V[2] = -vs, V[3] = vc;
}

}  // namespace

extern "C" {

// ---- wrapper.cpp:12-40 --------------------------------------------------------------------
void svd_2(double F00, double F01, double F10, double F11, double* U00, double* U01, double* U10, double* U11, double* s00,
           double* s01, double* s10, double* s11, double* V00, double* V01, double* V10, double* V11) {
    const double F[4] = {F00, F01, F10, F11};
    double U[4], s[2], V[4];
    svd2_givens(F, U, s, V);
    *U00 = U[0], *U01 = U[1], *U10 = U[2], *U11 = U[3];
    *s00 = s[0], *s01 = 0.0, *s10 = 0.0, *s11 = s[1];
    *V00 = V[0], *V01 = V[1], *V10 = V[2], *V11 = V[3];
}

void svd_3(double F00, double F01, double F02, double F10, double F11, double F12, double F20, double F21, double F22,
           double* U00, double* U01, double* U02, double* U10, double* U11, double* U12, double* U20, double* U21, double* U22,
           double* s00, double* s01, double* s02, double* s10, double* s11, double* s12, double* s20, double* s21, double* s22,
           double* V00, double* V01, double* V02, double* V10, double* V11, double* V12, double* V20, double* V21, double* V22) {
    const double F[9] = {F00, F01, F02, F10, F11, F12, F20, F21, F22};
    double U[9], s[3], V[9];
    svd3(F, U, s, V);
    double* const u[9] = {U00, U01, U02, U10, U11, U12, U20, U21, U22};
    double* const v[9] = {V00, V01, V02, V10, V11, V12, V20, V21, V22};
    double* const S[9] = {s00, s01, s02, s10, s11, s12, s20, s21, s22};
    for (int i = 0; i < 9; ++i) {
        *u[i] = U[i];
        *v[i] = V[i];
        *S[i] = (i % 4 == 0) ? s[i / 4] : 0.0;
    }
}

// ---- wrapper.cpp:42-88: project_pd_N(in_0 .. in_{N*N-1}, out_0 .. out_{N*N-1}) -------------
void project_pd_2(double in_0, double in_1, double in_2, double in_3, double* out_0, double* out_1, double* out_2,
                  double* out_3) {
    const double in[4] = {in_0, in_1, in_2, in_3};
    double* const out[4] = {out_0, out_1, out_2, out_3};
    project_pd_n(2, in, out);
}

void project_pd_3(double in_0, double in_1, double in_2, double in_3, double in_4, double in_5, double in_6,
                  double in_7, double in_8, double* out_0, double* out_1, double* out_2, double* out_3,
                  double* out_4, double* out_5, double* out_6, double* out_7, double* out_8) {
    const double in[9] = {in_0, in_1, in_2, in_3, in_4, in_5, in_6, in_7, in_8};
    double* const out[9] = {out_0, out_1, out_2, out_3, out_4, out_5, out_6, out_7, out_8};
    project_pd_n(3, in, out);
}

void project_pd_4(double in_0, double in_1, double in_2, double in_3, double in_4, double in_5, double in_6,
                  double in_7, double in_8, double in_9, double in_10, double in_11, double in_12, double in_13,
                  double in_14, double in_15, double* out_0, double* out_1, double* out_2, double* out_3,
                  double* out_4, double* out_5, double* out_6, double* out_7, double* out_8, double* out_9,
                  double* out_10, double* out_11, double* out_12, double* out_13, double* out_14, double* out_15) {
    const double in[16] = {in_0, in_1, in_2, in_3, in_4, in_5, in_6, in_7, in_8, in_9, in_10, in_11, in_12, in_13,
                         in_14, in_15};
    double* const out[16] = {out_0, out_1, out_2, out_3, out_4, out_5, out_6, out_7, out_8, out_9, out_10, out_11,
                             out_12, out_13, out_14, out_15};
    project_pd_n(4, in, out);
}

void project_pd_6(double in_0, double in_1, double in_2, double in_3, double in_4, double in_5, double in_6,
                  double in_7, double in_8, double in_9, double in_10, double in_11, double in_12, double in_13,
                  double in_14, double in_15, double in_16, double in_17, double in_18, double in_19, double in_20,
                  double in_21, double in_22, double in_23, double in_24, double in_25, double in_26, double in_27,
                  double in_28, double in_29, double in_30, double in_31, double in_32, double in_33, double in_34,
                  double in_35, double* out_0, double* out_1, double* out_2, double* out_3, double* out_4,
                  double* out_5, double* out_6, double* out_7, double* out_8, double* out_9, double* out_10,
                  double* out_11, double* out_12, double* out_13, double* out_14, double* out_15, double* out_16,
                  double* out_17, double* out_18, double* out_19, double* out_20, double* out_21, double* out_22,
                  double* out_23, double* out_24, double* out_25, double* out_26, double* out_27, double* out_28,
                  double* out_29, double* out_30, double* out_31, double* out_32, double* out_33, double* out_34,
                  double* out_35) {
    const double in[36] = {in_0, in_1, in_2, in_3, in_4, in_5, in_6, in_7, in_8, in_9, in_10, in_11, in_12, in_13,
                         in_14, in_15, in_16, in_17, in_18, in_19, in_20, in_21, in_22, in_23, in_24, in_25, in_26,
                         in_27, in_28, in_29, in_30, in_31, in_32, in_33, in_34, in_35};
    double* const out[36] = {out_0, out_1, out_2, out_3, out_4, out_5, out_6, out_7, out_8, out_9, out_10, out_11,
                             out_12, out_13, out_14, out_15, out_16, out_17, out_18, out_19, out_20, out_21, out_22,
                             out_23, out_24, out_25, out_26, out_27, out_28, out_29, out_30, out_31, out_32, out_33,
                             out_34, out_35};
    project_pd_n(6, in, out);
}

void project_pd_9(double in_0, double in_1, double in_2, double in_3, double in_4, double in_5, double in_6,
                  double in_7, double in_8, double in_9, double in_10, double in_11, double in_12, double in_13,
                  double in_14, double in_15, double in_16, double in_17, double in_18, double in_19, double in_20,
                  double in_21, double in_22, double in_23, double in_24, double in_25, double in_26, double in_27,
                  double in_28, double in_29, double in_30, double in_31, double in_32, double in_33, double in_34,
                  double in_35, double in_36, double in_37, double in_38, double in_39, double in_40, double in_41,
                  double in_42, double in_43, double in_44, double in_45, double in_46, double in_47, double in_48,
                  double in_49, double in_50, double in_51, double in_52, double in_53, double in_54, double in_55,
                  double in_56, double in_57, double in_58, double in_59, double in_60, double in_61, double in_62,
                  double in_63, double in_64, double in_65, double in_66, double in_67, double in_68, double in_69,
                  double in_70, double in_71, double in_72, double in_73, double in_74, double in_75, double in_76,
                  double in_77, double in_78, double in_79, double in_80, double* out_0, double* out_1,
                  double* out_2, double* out_3, double* out_4, double* out_5, double* out_6, double* out_7,
                  double* out_8, double* out_9, double* out_10, double* out_11, double* out_12, double* out_13,
                  double* out_14, double* out_15, double* out_16, double* out_17, double* out_18, double* out_19,
                  double* out_20, double* out_21, double* out_22, double* out_23, double* out_24, double* out_25,
                  double* out_26, double* out_27, double* out_28, double* out_29, double* out_30, double* out_31,
                  double* out_32, double* out_33, double* out_34, double* out_35, double* out_36, double* out_37,
                  double* out_38, double* out_39, double* out_40, double* out_41, double* out_42, double* out_43,
                  double* out_44, double* out_45, double* out_46, double* out_47, double* out_48, double* out_49,
                  double* out_50, double* out_51, double* out_52, double* out_53, double* out_54, double* out_55,
                  double* out_56, double* out_57, double* out_58, double* out_59, double* out_60, double* out_61,
                  double* out_62, double* out_63, double* out_64, double* out_65, double* out_66, double* out_67,
                  double* out_68, double* out_69, double* out_70, double* out_71, double* out_72, double* out_73,
                  double* out_74, double* out_75, double* out_76, double* out_77, double* out_78, double* out_79,
                  double* out_80) {
    const double in[81] = {in_0, in_1, in_2, in_3, in_4, in_5, in_6, in_7, in_8, in_9, in_10, in_11, in_12, in_13,
                         in_14, in_15, in_16, in_17, in_18, in_19, in_20, in_21, in_22, in_23, in_24, in_25, in_26,
                         in_27, in_28, in_29, in_30, in_31, in_32, in_33, in_34, in_35, in_36, in_37, in_38, in_39,
                         in_40, in_41, in_42, in_43, in_44, in_45, in_46, in_47, in_48, in_49, in_50, in_51, in_52,
                         in_53, in_54, in_55, in_56, in_57, in_58, in_59, in_60, in_61, in_62, in_63, in_64, in_65,
                         in_66, in_67, in_68, in_69, in_70, in_71, in_72, in_73, in_74, in_75, in_76, in_77, in_78,
                         in_79, in_80};
    double* const out[81] = {out_0, out_1, out_2, out_3, out_4, out_5, out_6, out_7, out_8, out_9, out_10, out_11,
                             out_12, out_13, out_14, out_15, out_16, out_17, out_18, out_19, out_20, out_21, out_22,
                             out_23, out_24, out_25, out_26, out_27, out_28, out_29, out_30, out_31, out_32, out_33,
                             out_34, out_35, out_36, out_37, out_38, out_39, out_40, out_41, out_42, out_43, out_44,
                             out_45, out_46, out_47, out_48, out_49, out_50, out_51, out_52, out_53, out_54, out_55,
                             out_56, out_57, out_58, out_59, out_60, out_61, out_62, out_63, out_64, out_65, out_66,
                             out_67, out_68, out_69, out_70, out_71, out_72, out_73, out_74, out_75, out_76, out_77,
                             out_78, out_79, out_80};
    project_pd_n(9, in, out);
}

void project_pd_12(double in_0, double in_1, double in_2, double in_3, double in_4, double in_5, double in_6,
                   double in_7, double in_8, double in_9, double in_10, double in_11, double in_12, double in_13,
                   double in_14, double in_15, double in_16, double in_17, double in_18, double in_19, double in_20,
                   double in_21, double in_22, double in_23, double in_24, double in_25, double in_26, double in_27,
                   double in_28, double in_29, double in_30, double in_31, double in_32, double in_33, double in_34,
                   double in_35, double in_36, double in_37, double in_38, double in_39, double in_40, double in_41,
                   double in_42, double in_43, double in_44, double in_45, double in_46, double in_47, double in_48,
                   double in_49, double in_50, double in_51, double in_52, double in_53, double in_54, double in_55,
                   double in_56, double in_57, double in_58, double in_59, double in_60, double in_61, double in_62,
                   double in_63, double in_64, double in_65, double in_66, double in_67, double in_68, double in_69,
                   double in_70, double in_71, double in_72, double in_73, double in_74, double in_75, double in_76,
                   double in_77, double in_78, double in_79, double in_80, double in_81, double in_82, double in_83,
                   double in_84, double in_85, double in_86, double in_87, double in_88, double in_89, double in_90,
                   double in_91, double in_92, double in_93, double in_94, double in_95, double in_96, double in_97,
                   double in_98, double in_99, double in_100, double in_101, double in_102, double in_103,
                   double in_104, double in_105, double in_106, double in_107, double in_108, double in_109,
                   double in_110, double in_111, double in_112, double in_113, double in_114, double in_115,
                   double in_116, double in_117, double in_118, double in_119, double in_120, double in_121,
                   double in_122, double in_123, double in_124, double in_125, double in_126, double in_127,
                   double in_128, double in_129, double in_130, double in_131, double in_132, double in_133,
                   double in_134, double in_135, double in_136, double in_137, double in_138, double in_139,
                   double in_140, double in_141, double in_142, double in_143, double* out_0, double* out_1,
                   double* out_2, double* out_3, double* out_4, double* out_5, double* out_6, double* out_7,
                   double* out_8, double* out_9, double* out_10, double* out_11, double* out_12, double* out_13,
                   double* out_14, double* out_15, double* out_16, double* out_17, double* out_18, double* out_19,
                   double* out_20, double* out_21, double* out_22, double* out_23, double* out_24, double* out_25,
                   double* out_26, double* out_27, double* out_28, double* out_29, double* out_30, double* out_31,
                   double* out_32, double* out_33, double* out_34, double* out_35, double* out_36, double* out_37,
                   double* out_38, double* out_39, double* out_40, double* out_41, double* out_42, double* out_43,
                   double* out_44, double* out_45, double* out_46, double* out_47, double* out_48, double* out_49,
                   double* out_50, double* out_51, double* out_52, double* out_53, double* out_54, double* out_55,
                   double* out_56, double* out_57, double* out_58, double* out_59, double* out_60, double* out_61,
                   double* out_62, double* out_63, double* out_64, double* out_65, double* out_66, double* out_67,
                   double* out_68, double* out_69, double* out_70, double* out_71, double* out_72, double* out_73,
                   double* out_74, double* out_75, double* out_76, double* out_77, double* out_78, double* out_79,
                   double* out_80, double* out_81, double* out_82, double* out_83, double* out_84, double* out_85,
                   double* out_86, double* out_87, double* out_88, double* out_89, double* out_90, double* out_91,
                   double* out_92, double* out_93, double* out_94, double* out_95, double* out_96, double* out_97,
                   double* out_98, double* out_99, double* out_100, double* out_101, double* out_102,
                   double* out_103, double* out_104, double* out_105, double* out_106, double* out_107,
                   double* out_108, double* out_109, double* out_110, double* out_111, double* out_112,
                   double* out_113, double* out_114, double* out_115, double* out_116, double* out_117,
                   double* out_118, double* out_119, double* out_120, double* out_121, double* out_122,
                   double* out_123, double* out_124, double* out_125, double* out_126, double* out_127,
                   double* out_128, double* out_129, double* out_130, double* out_131, double* out_132,
                   double* out_133, double* out_134, double* out_135, double* out_136, double* out_137,
                   double* out_138, double* out_139, double* out_140, double* out_141, double* out_142,
                   double* out_143) {
    const double in[144] = {in_0, in_1, in_2, in_3, in_4, in_5, in_6, in_7, in_8, in_9, in_10, in_11, in_12, in_13,
                         in_14, in_15, in_16, in_17, in_18, in_19, in_20, in_21, in_22, in_23, in_24, in_25, in_26,
                         in_27, in_28, in_29, in_30, in_31, in_32, in_33, in_34, in_35, in_36, in_37, in_38, in_39,
                         in_40, in_41, in_42, in_43, in_44, in_45, in_46, in_47, in_48, in_49, in_50, in_51, in_52,
                         in_53, in_54, in_55, in_56, in_57, in_58, in_59, in_60, in_61, in_62, in_63, in_64, in_65,
                         in_66, in_67, in_68, in_69, in_70, in_71, in_72, in_73, in_74, in_75, in_76, in_77, in_78,
                         in_79, in_80, in_81, in_82, in_83, in_84, in_85, in_86, in_87, in_88, in_89, in_90, in_91,
                         in_92, in_93, in_94, in_95, in_96, in_97, in_98, in_99, in_100, in_101, in_102, in_103,
                         in_104, in_105, in_106, in_107, in_108, in_109, in_110, in_111, in_112, in_113, in_114,
                         in_115, in_116, in_117, in_118, in_119, in_120, in_121, in_122, in_123, in_124, in_125,
                         in_126, in_127, in_128, in_129, in_130, in_131, in_132, in_133, in_134, in_135, in_136,
                         in_137, in_138, in_139, in_140, in_141, in_142, in_143};
    double* const out[144] = {out_0, out_1, out_2, out_3, out_4, out_5, out_6, out_7, out_8, out_9, out_10, out_11,
                             out_12, out_13, out_14, out_15, out_16, out_17, out_18, out_19, out_20, out_21, out_22,
                             out_23, out_24, out_25, out_26, out_27, out_28, out_29, out_30, out_31, out_32, out_33,
                             out_34, out_35, out_36, out_37, out_38, out_39, out_40, out_41, out_42, out_43, out_44,
                             out_45, out_46, out_47, out_48, out_49, out_50, out_51, out_52, out_53, out_54, out_55,
                             out_56, out_57, out_58, out_59, out_60, out_61, out_62, out_63, out_64, out_65, out_66,
                             out_67, out_68, out_69, out_70, out_71, out_72, out_73, out_74, out_75, out_76, out_77,
                             out_78, out_79, out_80, out_81, out_82, out_83, out_84, out_85, out_86, out_87, out_88,
                             out_89, out_90, out_91, out_92, out_93, out_94, out_95, out_96, out_97, out_98, out_99,
                             out_100, out_101, out_102, out_103, out_104, out_105, out_106, out_107, out_108,
                             out_109, out_110, out_111, out_112, out_113, out_114, out_115, out_116, out_117,
                             out_118, out_119, out_120, out_121, out_122, out_123, out_124, out_125, out_126,
                             out_127, out_128, out_129, out_130, out_131, out_132, out_133, out_134, out_135,
                             out_136, out_137, out_138, out_139, out_140, out_141, out_142, out_143};
    project_pd_n(12, in, out);
}

// ---- wrapper.cpp:90-198: solve_N(in_0 .. in_{N*N-1}, rhs_0 .. rhs_{N-1}, out_0 .. out_{N-1}) -
void solve_2(double in_0, double in_1, double in_2, double in_3, double rhs_0, double rhs_1, double* out_0,
             double* out_1) {
    const double in[4] = {in_0, in_1, in_2, in_3};
    const double rhs[2] = {rhs_0, rhs_1};
    double* const out[2] = {out_0, out_1};
    double x[2];
    solve_n(2, in, rhs, x);
    for (int i = 0; i < 2; ++i) *out[i] = x[i];
}

void solve_3(double in_0, double in_1, double in_2, double in_3, double in_4, double in_5, double in_6, double in_7,
             double in_8, double rhs_0, double rhs_1, double rhs_2, double* out_0, double* out_1, double* out_2) {
    const double in[9] = {in_0, in_1, in_2, in_3, in_4, in_5, in_6, in_7, in_8};
    const double rhs[3] = {rhs_0, rhs_1, rhs_2};
    double* const out[3] = {out_0, out_1, out_2};
    double x[3];
    solve_n(3, in, rhs, x);
    for (int i = 0; i < 3; ++i) *out[i] = x[i];
}

void solve_4(double in_0, double in_1, double in_2, double in_3, double in_4, double in_5, double in_6, double in_7,
             double in_8, double in_9, double in_10, double in_11, double in_12, double in_13, double in_14,
             double in_15, double rhs_0, double rhs_1, double rhs_2, double rhs_3, double* out_0, double* out_1,
             double* out_2, double* out_3) {
    const double in[16] = {in_0, in_1, in_2, in_3, in_4, in_5, in_6, in_7, in_8, in_9, in_10, in_11, in_12, in_13,
                         in_14, in_15};
    const double rhs[4] = {rhs_0, rhs_1, rhs_2, rhs_3};
    double* const out[4] = {out_0, out_1, out_2, out_3};
    double x[4];
    solve_n(4, in, rhs, x);
    for (int i = 0; i < 4; ++i) *out[i] = x[i];
}

void solve_6(double in_0, double in_1, double in_2, double in_3, double in_4, double in_5, double in_6, double in_7,
             double in_8, double in_9, double in_10, double in_11, double in_12, double in_13, double in_14,
             double in_15, double in_16, double in_17, double in_18, double in_19, double in_20, double in_21,
             double in_22, double in_23, double in_24, double in_25, double in_26, double in_27, double in_28,
             double in_29, double in_30, double in_31, double in_32, double in_33, double in_34, double in_35,
             double rhs_0, double rhs_1, double rhs_2, double rhs_3, double rhs_4, double rhs_5, double* out_0,
             double* out_1, double* out_2, double* out_3, double* out_4, double* out_5) {
    const double in[36] = {in_0, in_1, in_2, in_3, in_4, in_5, in_6, in_7, in_8, in_9, in_10, in_11, in_12, in_13,
                         in_14, in_15, in_16, in_17, in_18, in_19, in_20, in_21, in_22, in_23, in_24, in_25, in_26,
                         in_27, in_28, in_29, in_30, in_31, in_32, in_33, in_34, in_35};
    const double rhs[6] = {rhs_0, rhs_1, rhs_2, rhs_3, rhs_4, rhs_5};
    double* const out[6] = {out_0, out_1, out_2, out_3, out_4, out_5};
    double x[6];
    solve_n(6, in, rhs, x);
    for (int i = 0; i < 6; ++i) *out[i] = x[i];
}

void solve_9(double in_0, double in_1, double in_2, double in_3, double in_4, double in_5, double in_6, double in_7,
             double in_8, double in_9, double in_10, double in_11, double in_12, double in_13, double in_14,
             double in_15, double in_16, double in_17, double in_18, double in_19, double in_20, double in_21,
             double in_22, double in_23, double in_24, double in_25, double in_26, double in_27, double in_28,
             double in_29, double in_30, double in_31, double in_32, double in_33, double in_34, double in_35,
             double in_36, double in_37, double in_38, double in_39, double in_40, double in_41, double in_42,
             double in_43, double in_44, double in_45, double in_46, double in_47, double in_48, double in_49,
             double in_50, double in_51, double in_52, double in_53, double in_54, double in_55, double in_56,
             double in_57, double in_58, double in_59, double in_60, double in_61, double in_62, double in_63,
             double in_64, double in_65, double in_66, double in_67, double in_68, double in_69, double in_70,
             double in_71, double in_72, double in_73, double in_74, double in_75, double in_76, double in_77,
             double in_78, double in_79, double in_80, double rhs_0, double rhs_1, double rhs_2, double rhs_3,
             double rhs_4, double rhs_5, double rhs_6, double rhs_7, double rhs_8, double* out_0, double* out_1,
             double* out_2, double* out_3, double* out_4, double* out_5, double* out_6, double* out_7, double* out_8) {
    const double in[81] = {in_0, in_1, in_2, in_3, in_4, in_5, in_6, in_7, in_8, in_9, in_10, in_11, in_12, in_13,
                         in_14, in_15, in_16, in_17, in_18, in_19, in_20, in_21, in_22, in_23, in_24, in_25, in_26,
                         in_27, in_28, in_29, in_30, in_31, in_32, in_33, in_34, in_35, in_36, in_37, in_38, in_39,
                         in_40, in_41, in_42, in_43, in_44, in_45, in_46, in_47, in_48, in_49, in_50, in_51, in_52,
                         in_53, in_54, in_55, in_56, in_57, in_58, in_59, in_60, in_61, in_62, in_63, in_64, in_65,
                         in_66, in_67, in_68, in_69, in_70, in_71, in_72, in_73, in_74, in_75, in_76, in_77, in_78,
                         in_79, in_80};
    const double rhs[9] = {rhs_0, rhs_1, rhs_2, rhs_3, rhs_4, rhs_5, rhs_6, rhs_7, rhs_8};
    double* const out[9] = {out_0, out_1, out_2, out_3, out_4, out_5, out_6, out_7, out_8};
    double x[9];
    solve_n(9, in, rhs, x);
    for (int i = 0; i < 9; ++i) *out[i] = x[i];
}
// ---- wrapper.cpp:200-252 ------------------------------------------------------------------
void get_smallest_positive_real_quad_root(double a, double b, double c, double tol, double* ret) {
    *ret = quad_root_pos(a, b, c, tol);
}

void get_smallest_positive_real_cubic_root(double a, double b, double c, double d, double tol, double* ret) {
    *ret = cubic_root_pos(a, b, c, d, tol);
}

// ---- wrapper.cpp:254-328 ------------------------------------------------------------------
void point_triangle_ccd(double p0, double p1, double p2, double t00, double t01, double t02, double t10, double t11, double t12,
                        double t20, double t21, double t22, double dp0, double dp1, double dp2, double dt00, double dt01,
                        double dt02, double dt10, double dt11, double dt12, double dt20, double dt21, double dt22, double eta,
                        double dist2_cur, double* ret) {
    *ret = pt_ccd(mk(p0, p1, p2), mk(t00, t01, t02), mk(t10, t11, t12), mk(t20, t21, t22), mk(dp0, dp1, dp2), mk(dt00, dt01, dt02),
                  mk(dt10, dt11, dt12), mk(dt20, dt21, dt22), eta, dist2_cur);
}

void edge_edge_ccd(double a00, double a01, double a02, double a10, double a11, double a12, double b00, double b01, double b02,
                   double b10, double b11, double b12, double da00, double da01, double da02, double da10, double da11, double da12,
                   double db00, double db01, double db02, double db10, double db11, double db12, double eta, double dist2_cur,
                   double* ret) {
    *ret = ee_ccd(mk(a00, a01, a02), mk(a10, a11, a12), mk(b00, b01, b02), mk(b10, b11, b12), mk(da00, da01, da02),
                  mk(da10, da11, da12), mk(db00, db01, db02), mk(db10, db11, db12), eta, dist2_cur);
}

}  // extern "C"

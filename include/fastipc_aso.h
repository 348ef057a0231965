/*
 * libfastipc — host-side scalar functions with the signatures of the reference's native library
 * a.so (common/math/wrapper/wrapper.cpp, FastIPC checkout), so that the reference's own ctypes
 * glue (common/math/external_func.py:4, common/math/math_tools.py:78-181, common/math/ipc.py:
 * 382-411) can load libfastipc.so in place of a.so.  Inputs are doubles by value, outputs double*
 * slots; no status codes, no allocation, no global state (reentrant).  They run on the calling
 * CPU thread and need no GPU.  Differences from a.so, all within the reference's own rounding:
 *  - svd_3 returns the same singular values; its singular vectors may differ from the
 *    reference's by a sign shared by a column of U and the same column of V;
 *  - solve_N reproduces the reference's pivoted LDL^T with pivots raised to 1e-8; where that
 *    raise happens (indefinite input) the system is ill-conditioned and results agree only to
 *    the rounding its condition number allows.
 */
#ifndef FASTIPC_ASO_H
#define FASTIPC_ASO_H

#ifdef __cplusplus
extern "C" {
#endif

/* wrapper.cpp:12-25 */
void svd_2(double F00, double F01, double F10, double F11, double* U00, double* U01, double* U10,
           double* U11, double* s00, double* s01, double* s10, double* s11, double* V00, double* V01,
           double* V10, double* V11);

/* wrapper.cpp:27-40 */
void svd_3(double F00, double F01, double F02, double F10, double F11, double F12, double F20, double F21,
           double F22, double* U00, double* U01, double* U02, double* U10, double* U11, double* U12,
           double* U20, double* U21, double* U22, double* s00, double* s01, double* s02, double* s10,
           double* s11, double* s12, double* s20, double* s21, double* s22, double* V00, double* V01,
           double* V02, double* V10, double* V11, double* V12, double* V20, double* V21, double* V22);

/* wrapper.cpp:42-48 */
void project_pd_2(double in_0, double in_1, double in_2, double in_3, double* out_0, double* out_1,
                  double* out_2, double* out_3);

/* wrapper.cpp:50-56 */
void project_pd_3(double in_0, double in_1, double in_2, double in_3, double in_4, double in_5, double in_6,
                  double in_7, double in_8, double* out_0, double* out_1, double* out_2, double* out_3,
                  double* out_4, double* out_5, double* out_6, double* out_7, double* out_8);

/* wrapper.cpp:58-64 */
void project_pd_4(double in_0, double in_1, double in_2, double in_3, double in_4, double in_5, double in_6,
                  double in_7, double in_8, double in_9, double in_10, double in_11, double in_12,
                  double in_13, double in_14, double in_15, double* out_0, double* out_1, double* out_2,
                  double* out_3, double* out_4, double* out_5, double* out_6, double* out_7, double* out_8,
                  double* out_9, double* out_10, double* out_11, double* out_12, double* out_13,
                  double* out_14, double* out_15);

/* wrapper.cpp:66-72 */
void project_pd_6(double in_0, double in_1, double in_2, double in_3, double in_4, double in_5, double in_6,
                  double in_7, double in_8, double in_9, double in_10, double in_11, double in_12,
                  double in_13, double in_14, double in_15, double in_16, double in_17, double in_18,
                  double in_19, double in_20, double in_21, double in_22, double in_23, double in_24,
                  double in_25, double in_26, double in_27, double in_28, double in_29, double in_30,
                  double in_31, double in_32, double in_33, double in_34, double in_35, double* out_0,
                  double* out_1, double* out_2, double* out_3, double* out_4, double* out_5, double* out_6,
                  double* out_7, double* out_8, double* out_9, double* out_10, double* out_11,
                  double* out_12, double* out_13, double* out_14, double* out_15, double* out_16,
                  double* out_17, double* out_18, double* out_19, double* out_20, double* out_21,
                  double* out_22, double* out_23, double* out_24, double* out_25, double* out_26,
                  double* out_27, double* out_28, double* out_29, double* out_30, double* out_31,
                  double* out_32, double* out_33, double* out_34, double* out_35);

/* wrapper.cpp:74-80 */
void project_pd_9(double in_0, double in_1, double in_2, double in_3, double in_4, double in_5, double in_6,
                  double in_7, double in_8, double in_9, double in_10, double in_11, double in_12,
                  double in_13, double in_14, double in_15, double in_16, double in_17, double in_18,
                  double in_19, double in_20, double in_21, double in_22, double in_23, double in_24,
                  double in_25, double in_26, double in_27, double in_28, double in_29, double in_30,
                  double in_31, double in_32, double in_33, double in_34, double in_35, double in_36,
                  double in_37, double in_38, double in_39, double in_40, double in_41, double in_42,
                  double in_43, double in_44, double in_45, double in_46, double in_47, double in_48,
                  double in_49, double in_50, double in_51, double in_52, double in_53, double in_54,
                  double in_55, double in_56, double in_57, double in_58, double in_59, double in_60,
                  double in_61, double in_62, double in_63, double in_64, double in_65, double in_66,
                  double in_67, double in_68, double in_69, double in_70, double in_71, double in_72,
                  double in_73, double in_74, double in_75, double in_76, double in_77, double in_78,
                  double in_79, double in_80, double* out_0, double* out_1, double* out_2, double* out_3,
                  double* out_4, double* out_5, double* out_6, double* out_7, double* out_8, double* out_9,
                  double* out_10, double* out_11, double* out_12, double* out_13, double* out_14,
                  double* out_15, double* out_16, double* out_17, double* out_18, double* out_19,
                  double* out_20, double* out_21, double* out_22, double* out_23, double* out_24,
                  double* out_25, double* out_26, double* out_27, double* out_28, double* out_29,
                  double* out_30, double* out_31, double* out_32, double* out_33, double* out_34,
                  double* out_35, double* out_36, double* out_37, double* out_38, double* out_39,
                  double* out_40, double* out_41, double* out_42, double* out_43, double* out_44,
                  double* out_45, double* out_46, double* out_47, double* out_48, double* out_49,
                  double* out_50, double* out_51, double* out_52, double* out_53, double* out_54,
                  double* out_55, double* out_56, double* out_57, double* out_58, double* out_59,
                  double* out_60, double* out_61, double* out_62, double* out_63, double* out_64,
                  double* out_65, double* out_66, double* out_67, double* out_68, double* out_69,
                  double* out_70, double* out_71, double* out_72, double* out_73, double* out_74,
                  double* out_75, double* out_76, double* out_77, double* out_78, double* out_79,
                  double* out_80);

/* wrapper.cpp:82-88 */
void project_pd_12(double in_0, double in_1, double in_2, double in_3, double in_4, double in_5, double in_6,
                   double in_7, double in_8, double in_9, double in_10, double in_11, double in_12,
                   double in_13, double in_14, double in_15, double in_16, double in_17, double in_18,
                   double in_19, double in_20, double in_21, double in_22, double in_23, double in_24,
                   double in_25, double in_26, double in_27, double in_28, double in_29, double in_30,
                   double in_31, double in_32, double in_33, double in_34, double in_35, double in_36,
                   double in_37, double in_38, double in_39, double in_40, double in_41, double in_42,
                   double in_43, double in_44, double in_45, double in_46, double in_47, double in_48,
                   double in_49, double in_50, double in_51, double in_52, double in_53, double in_54,
                   double in_55, double in_56, double in_57, double in_58, double in_59, double in_60,
                   double in_61, double in_62, double in_63, double in_64, double in_65, double in_66,
                   double in_67, double in_68, double in_69, double in_70, double in_71, double in_72,
                   double in_73, double in_74, double in_75, double in_76, double in_77, double in_78,
                   double in_79, double in_80, double in_81, double in_82, double in_83, double in_84,
                   double in_85, double in_86, double in_87, double in_88, double in_89, double in_90,
                   double in_91, double in_92, double in_93, double in_94, double in_95, double in_96,
                   double in_97, double in_98, double in_99, double in_100, double in_101, double in_102,
                   double in_103, double in_104, double in_105, double in_106, double in_107, double in_108,
                   double in_109, double in_110, double in_111, double in_112, double in_113, double in_114,
                   double in_115, double in_116, double in_117, double in_118, double in_119, double in_120,
                   double in_121, double in_122, double in_123, double in_124, double in_125, double in_126,
                   double in_127, double in_128, double in_129, double in_130, double in_131, double in_132,
                   double in_133, double in_134, double in_135, double in_136, double in_137, double in_138,
                   double in_139, double in_140, double in_141, double in_142, double in_143, double* out_0,
                   double* out_1, double* out_2, double* out_3, double* out_4, double* out_5, double* out_6,
                   double* out_7, double* out_8, double* out_9, double* out_10, double* out_11,
                   double* out_12, double* out_13, double* out_14, double* out_15, double* out_16,
                   double* out_17, double* out_18, double* out_19, double* out_20, double* out_21,
                   double* out_22, double* out_23, double* out_24, double* out_25, double* out_26,
                   double* out_27, double* out_28, double* out_29, double* out_30, double* out_31,
                   double* out_32, double* out_33, double* out_34, double* out_35, double* out_36,
                   double* out_37, double* out_38, double* out_39, double* out_40, double* out_41,
                   double* out_42, double* out_43, double* out_44, double* out_45, double* out_46,
                   double* out_47, double* out_48, double* out_49, double* out_50, double* out_51,
                   double* out_52, double* out_53, double* out_54, double* out_55, double* out_56,
                   double* out_57, double* out_58, double* out_59, double* out_60, double* out_61,
                   double* out_62, double* out_63, double* out_64, double* out_65, double* out_66,
                   double* out_67, double* out_68, double* out_69, double* out_70, double* out_71,
                   double* out_72, double* out_73, double* out_74, double* out_75, double* out_76,
                   double* out_77, double* out_78, double* out_79, double* out_80, double* out_81,
                   double* out_82, double* out_83, double* out_84, double* out_85, double* out_86,
                   double* out_87, double* out_88, double* out_89, double* out_90, double* out_91,
                   double* out_92, double* out_93, double* out_94, double* out_95, double* out_96,
                   double* out_97, double* out_98, double* out_99, double* out_100, double* out_101,
                   double* out_102, double* out_103, double* out_104, double* out_105, double* out_106,
                   double* out_107, double* out_108, double* out_109, double* out_110, double* out_111,
                   double* out_112, double* out_113, double* out_114, double* out_115, double* out_116,
                   double* out_117, double* out_118, double* out_119, double* out_120, double* out_121,
                   double* out_122, double* out_123, double* out_124, double* out_125, double* out_126,
                   double* out_127, double* out_128, double* out_129, double* out_130, double* out_131,
                   double* out_132, double* out_133, double* out_134, double* out_135, double* out_136,
                   double* out_137, double* out_138, double* out_139, double* out_140, double* out_141,
                   double* out_142, double* out_143);

/* wrapper.cpp:90-110 */
void solve_2(double in_0, double in_1, double in_2, double in_3, double rhs_0, double rhs_1, double* out_0,
             double* out_1);

/* wrapper.cpp:112-132 */
void solve_3(double in_0, double in_1, double in_2, double in_3, double in_4, double in_5, double in_6,
             double in_7, double in_8, double rhs_0, double rhs_1, double rhs_2, double* out_0,
             double* out_1, double* out_2);

/* wrapper.cpp:134-154 */
void solve_4(double in_0, double in_1, double in_2, double in_3, double in_4, double in_5, double in_6,
             double in_7, double in_8, double in_9, double in_10, double in_11, double in_12, double in_13,
             double in_14, double in_15, double rhs_0, double rhs_1, double rhs_2, double rhs_3,
             double* out_0, double* out_1, double* out_2, double* out_3);

/* wrapper.cpp:156-176 */
void solve_6(double in_0, double in_1, double in_2, double in_3, double in_4, double in_5, double in_6,
             double in_7, double in_8, double in_9, double in_10, double in_11, double in_12, double in_13,
             double in_14, double in_15, double in_16, double in_17, double in_18, double in_19,
             double in_20, double in_21, double in_22, double in_23, double in_24, double in_25,
             double in_26, double in_27, double in_28, double in_29, double in_30, double in_31,
             double in_32, double in_33, double in_34, double in_35, double rhs_0, double rhs_1,
             double rhs_2, double rhs_3, double rhs_4, double rhs_5, double* out_0, double* out_1,
             double* out_2, double* out_3, double* out_4, double* out_5);

/* wrapper.cpp:178-198 */
void solve_9(double in_0, double in_1, double in_2, double in_3, double in_4, double in_5, double in_6,
             double in_7, double in_8, double in_9, double in_10, double in_11, double in_12, double in_13,
             double in_14, double in_15, double in_16, double in_17, double in_18, double in_19,
             double in_20, double in_21, double in_22, double in_23, double in_24, double in_25,
             double in_26, double in_27, double in_28, double in_29, double in_30, double in_31,
             double in_32, double in_33, double in_34, double in_35, double in_36, double in_37,
             double in_38, double in_39, double in_40, double in_41, double in_42, double in_43,
             double in_44, double in_45, double in_46, double in_47, double in_48, double in_49,
             double in_50, double in_51, double in_52, double in_53, double in_54, double in_55,
             double in_56, double in_57, double in_58, double in_59, double in_60, double in_61,
             double in_62, double in_63, double in_64, double in_65, double in_66, double in_67,
             double in_68, double in_69, double in_70, double in_71, double in_72, double in_73,
             double in_74, double in_75, double in_76, double in_77, double in_78, double in_79,
             double in_80, double rhs_0, double rhs_1, double rhs_2, double rhs_3, double rhs_4,
             double rhs_5, double rhs_6, double rhs_7, double rhs_8, double* out_0, double* out_1,
             double* out_2, double* out_3, double* out_4, double* out_5, double* out_6, double* out_7,
             double* out_8);

/* wrapper.cpp:200-218 */
void get_smallest_positive_real_quad_root(double a, double b, double c, double tol, double* ret);

/* wrapper.cpp:220-252 */
void get_smallest_positive_real_cubic_root(double a, double b, double c, double d, double tol, double* ret);

/* wrapper.cpp:254-290 */
void point_triangle_ccd(double p0, double p1, double p2, double t00, double t01, double t02, double t10,
                        double t11, double t12, double t20, double t21, double t22, double dp0, double dp1,
                        double dp2, double dt00, double dt01, double dt02, double dt10, double dt11,
                        double dt12, double dt20, double dt21, double dt22, double eta, double dist2_cur,
                        double* ret);

/* wrapper.cpp:292-328 */
void edge_edge_ccd(double a00, double a01, double a02, double a10, double a11, double a12, double b00,
                   double b01, double b02, double b10, double b11, double b12, double da00, double da01,
                   double da02, double da10, double da11, double da12, double db00, double db01, double db02,
                   double db10, double db11, double db12, double eta, double dist2_cur, double* ret);

#ifdef __cplusplus
}
#endif

#endif

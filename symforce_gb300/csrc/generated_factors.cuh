// Generated by `python -m symforce_gb300.codegen --write` from the sympy residuals in
// symforce_gb300/factor_defs.py; do not edit by hand.
#pragma once

namespace sfg {

// SFG_FACTOR_PRIOR_ROT3: diag(s) Log(prior^-1 x)
// Generated by symforce_gb300.codegen from a sympy residual: 3 residual rows, tangent
// dimension 3; residual in FP64, Jacobian (row-major) in T.
struct GenPriorRot3 {
  static constexpr int NK = 1, NC = 8, RD = 3, TD = 3, MK = 0;
  static constexpr int kTangent[NK] = {3};
  static constexpr int kStorage[NK] = {4};
  static constexpr SFG_HD int KT(int k) { return (k == 0 ? 3 : 0); }
  static constexpr SFG_HD int KS(int k) { return (k == 0 ? 4 : 0); }
  template <typename T>
  static SFG_HD void Run(const double* const* x, const double* c, double* r, T* J) {
    const double t0 = c[0]*x[0][0] + c[1]*x[0][1] + c[2]*x[0][2] + c[3]*x[0][3];
    const double t1 = t0 >= 0;
    const double t2 = ((t1) ? (
   1
)
: (
   -1
));
    const double t3 = c[4]*t2;
    const double t4 = c[0]*x[0][3] + c[1]*x[0][2] - c[2]*x[0][1] - c[3]*x[0][0];
    const double t5 = c[7] - 1;
    const double t6 = -t5;
    const double t7 = ((t1) ? (
   c[7] > 1 - t0
)
: (
   c[7] > t0 + 1
));
    const double t8 = pow(t0, 2);
    const double t9 = ((t7) ? (
   pow(t6, 2)
)
: (
   t8
)) - 1;
    const double t10 = -t9;
    const double t11 = pow(t10, -1.0/2.0);
    const double t12 = acos(((t7) ? (
   t6
)
: (
   ((t1) ? (
      t0
   )
   : (
      -t0
   ))
)));
    const double t13 = t11*t12;
    const double t14 = t13*t4;
    const double t15 = c[0]*x[0][2] - c[1]*x[0][3] - c[2]*x[0][0] + c[3]*x[0][1];
    const double t16 = t13*t15;
    const double t17 = c[5]*t2;
    const double t18 = c[0]*x[0][1] - c[1]*x[0][0] + c[2]*x[0][3] - c[3]*x[0][2];
    const double t19 = t13*t18;
    const double t20 = c[6]*t2;
    const double t21 = -t0*t11*t12;
    const double t22 = 2*((t7) ? (
   0
)
: (
   ((t1) ? (
      (1.0/2.0)*t4
   )
   : (
      -1.0/2.0*t4
   ))
));
    const double t23 = 1.0/t9;
    const double t24 = t23*t4;
    const double t25 = ((t7) ? (
   0
)
: (
   t0*t4
));
    const double t26 = t12/pow(t10, 3.0/2.0);
    const double t27 = t26*t4;
    const double t28 = ((t7) ? (
   0
)
: (
   ((t1) ? (
      -1.0/2.0*t15
   )
   : (
      (1.0/2.0)*t15
   ))
));
    const double t29 = 2*t24;
    const double t30 = -t19;
    const double t31 = ((t7) ? (
   0
)
: (
   -t0*t15
));
    const double t32 = ((t7) ? (
   0
)
: (
   ((t1) ? (
      (1.0/2.0)*t18
   )
   : (
      -1.0/2.0*t18
   ))
));
    const double t33 = ((t7) ? (
   0
)
: (
   t0*t18
));
    const double t34 = t15/(((t7) ? (
   pow(t5, 2)
)
: (
   t8
)) - 1);
    const double t35 = t15*t26;
    const double t36 = 2*t34;
    const double t37 = t18*t23;
    const double t38 = t18*t26;
    const double t39 = 2*t37;
    r[0] = -2*t14*t3;
    r[1] = 2*t16*t17;
    r[2] = -2*t19*t20;
    J[0] = T(t3*(-t21 - t22*t24 - t25*t27));
    J[1] = T(t3*(-t27*t31 - t28*t29 - t30));
    J[2] = T(t3*(t11*t12*t15 - t27*t33 - t29*t32));
    J[3] = T(t17*(t22*t34 + t25*t35 + t30));
    J[4] = T(t17*(t0*t13 + t28*t36 + t31*t35));
    J[5] = T(t17*(t14 + t32*t36 + t33*t35));
    J[6] = T(-t20*(t16 + t22*t37 + t25*t38));
    J[7] = T(-t20*(t14 + t28*t39 + t31*t38));
    J[8] = T(t20*(-t21 - t32*t39 - t33*t38));
  }
};

// SFG_FACTOR_BETWEEN_ROT3: diag(s) Log(a_T_b^-1 a^-1 b)
// Generated by symforce_gb300.codegen from a sympy residual: 3 residual rows, tangent
// dimension 6; residual in FP64, Jacobian (row-major) in T.
struct GenBetweenRot3 {
  static constexpr int NK = 2, NC = 8, RD = 3, TD = 6, MK = 0;
  static constexpr int kTangent[NK] = {3, 3};
  static constexpr int kStorage[NK] = {4, 4};
  static constexpr SFG_HD int KT(int k) { return (k == 0 ? 3 : (k == 1 ? 3 : 0)); }
  static constexpr SFG_HD int KS(int k) { return (k == 0 ? 4 : (k == 1 ? 4 : 0)); }
  template <typename T>
  static SFG_HD void Run(const double* const* x, const double* c, double* r, T* J) {
    const double t0 = x[0][0]*x[1][1] - x[0][1]*x[1][0] + x[0][2]*x[1][3] - x[0][3]*x[1][2];
    const double t1 = c[2]*t0;
    const double t2 = x[0][0]*x[1][2] - x[0][1]*x[1][3] - x[0][2]*x[1][0] + x[0][3]*x[1][1];
    const double t3 = c[1]*t2;
    const double t4 = -t3;
    const double t5 = x[0][0]*x[1][3] + x[0][1]*x[1][2] - x[0][2]*x[1][1] - x[0][3]*x[1][0];
    const double t6 = c[0]*t5;
    const double t7 = x[0][0]*x[1][0] + x[0][1]*x[1][1] + x[0][2]*x[1][2] + x[0][3]*x[1][3];
    const double t8 = c[3]*t7;
    const double t9 = t6 - t8;
    const double t10 = t1 + t4 + t9;
    const double t11 = t10 <= 0;
    const double t12 = ((t11) ? (
   1
)
: (
   -1
));
    const double t13 = c[4]*t12;
    const double t14 = c[3]*t5;
    const double t15 = c[1]*t0;
    const double t16 = -t15;
    const double t17 = c[0]*t7;
    const double t18 = c[2]*t2;
    const double t19 = t17 - t18;
    const double t20 = t14 + t16 + t19;
    const double t21 = c[7] - 1;
    const double t22 = -t21;
    const double t23 = -t0;
    const double t24 = c[2]*t23;
    const double t25 = -t5;
    const double t26 = c[0]*t25 + t8;
    const double t27 = t24 + t26 + t3;
    const double t28 = c[7] > 1 - t27;
    const double t29 = pow(t27, 2);
    const double t30 = ((((t27 >= 0) ? (
   t28
)
: (
   c[7] > t27 + 1
))) ? (
   pow(t22, 2)
)
: (
   t29
)) - 1;
    const double t31 = -t30;
    const double t32 = pow(t31, -1.0/2.0);
    const double t33 = c[7] > -t1 + t3 - t6 + t8 + 1;
    const double t34 = ((t11) ? (
   c[7] > t10 + 1
)
: (
   t33
));
    const double t35 = -t10;
    const double t36 = acos(((t34) ? (
   t22
)
: (
   ((t11) ? (
      t35
   )
   : (
      t10
   ))
)));
    const double t37 = t32*t36;
    const double t38 = c[5]*t12;
    const double t39 = c[1]*t7;
    const double t40 = c[3]*t2;
    const double t41 = c[0]*t0;
    const double t42 = c[2]*t5;
    const double t43 = t41 - t42;
    const double t44 = t39 - t40 + t43;
    const double t45 = 2*t44;
    const double t46 = c[1]*t5;
    const double t47 = c[3]*t0;
    const double t48 = c[0]*t2;
    const double t49 = c[2]*t7;
    const double t50 = t48 + t49;
    const double t51 = t46 + t47 + t50;
    const double t52 = t37*t51;
    const double t53 = c[6]*t12;
    const double t54 = ((t11) ? (
   t28
)
: (
   t33
));
    const double t55 = t14 + t17;
    const double t56 = t15 + t18 + t55;
    const double t57 = (1.0/2.0)*t56;
    const double t58 = -t57;
    const double t59 = c[3]*t25;
    const double t60 = c[1]*t23;
    const double t61 = -t2;
    const double t62 = c[2]*t61;
    const double t63 = t60 + t62;
    const double t64 = -t17 + t59 + t63;
    const double t65 = ((t54) ? (
   0
)
: (
   ((t11) ? (
      t58
   )
   : (
      -1.0/2.0*t64
   ))
));
    const double t66 = -t59;
    const double t67 = t19 + t60 + t66;
    const double t68 = 2/t30;
    const double t69 = t67*t68;
    const double t70 = c[1]*t61 - t24;
    const double t71 = acos(((t54) ? (
   t22
)
: (
   ((t11) ? (
      t35
   )
   : (
      -t27
   ))
)));
    const double t72 = t32*t71;
    const double t73 = -t35*t56;
    const double t74 = ((t54) ? (
   0
)
: (
   ((t11) ? (
      t73
   )
   : (
      t27*t64
   ))
));
    const double t75 = pow(t31, -3.0/2.0);
    const double t76 = t71*t75;
    const double t77 = t67*t76;
    const double t78 = c[1]*t25;
    const double t79 = -t47;
    const double t80 = t78 + t79;
    const double t81 = -t39;
    const double t82 = t40 + t81;
    const double t83 = t43 + t82;
    const double t84 = (1.0/2.0)*t83;
    const double t85 = c[2]*t25;
    const double t86 = t41 + t85;
    const double t87 = t82 + t86;
    const double t88 = ((t54) ? (
   0
)
: (
   ((t11) ? (
      t84
   )
   : (
      -1.0/2.0*t87
   ))
));
    const double t89 = t35*t83;
    const double t90 = ((t54) ? (
   0
)
: (
   ((t11) ? (
      t89
   )
   : (
      t27*t87
   ))
));
    const double t91 = -t49;
    const double t92 = t48 + t91;
    const double t93 = t46 + t92;
    const double t94 = t79 + t93;
    const double t95 = (1.0/2.0)*t94;
    const double t96 = c[3]*t23;
    const double t97 = t93 + t96;
    const double t98 = ((t54) ? (
   0
)
: (
   ((t11) ? (
      t95
   )
   : (
      -1.0/2.0*t97
   ))
));
    const double t99 = t35*t94;
    const double t100 = ((t54) ? (
   0
)
: (
   ((t11) ? (
      t99
   )
   : (
      t27*t97
   ))
));
    const double t101 = (1.0/2.0)*t20;
    const double t102 = t55 + t63;
    const double t103 = ((t54) ? (
   0
)
: (
   ((t11) ? (
      t101
   )
   : (
      -1.0/2.0*t102
   ))
));
    const double t104 = t20*t35;
    const double t105 = ((t54) ? (
   0
)
: (
   ((t11) ? (
      t104
   )
   : (
      t102*t27
   ))
));
    const double t106 = (1.0/2.0)*t44;
    const double t107 = c[3]*t61;
    const double t108 = t107 + t39 + t86;
    const double t109 = ((t54) ? (
   0
)
: (
   ((t11) ? (
      t106
   )
   : (
      -1.0/2.0*t108
   ))
));
    const double t110 = t35*t44;
    const double t111 = ((t54) ? (
   0
)
: (
   ((t11) ? (
      t110
   )
   : (
      t108*t27
   ))
));
    const double t112 = (1.0/2.0)*t51;
    const double t113 = ((t11) ? (
   t112
)
: (
   -t112
));
    const double t114 = ((t54) ? (
   0
)
: (
   t113
));
    const double t115 = t35*t51;
    const double t116 = ((t54) ? (
   0
)
: (
   ((t11) ? (
      t115
   )
   : (
      t27*t51
   ))
));
    const double t117 = t45/(((t54) ? (
   pow(t21, 2)
)
: (
   ((t11) ? (
      pow(t35, 2)
   )
   : (
      t29
   ))
)) - 1);
    const double t118 = t36*t44*t75;
    const double t119 = t6 + t8;
    const double t120 = t16 + t17;
    const double t121 = t50 - t78 - t96;
    const double t122 = t121*t68;
    const double t123 = c[0]*t23 - t107;
    const double t124 = t121*t76;
    r[0] = -2*t13*t20*t37;
    r[1] = -t37*t38*t45;
    r[2] = -2*t52*t53;
    J[0] = T(-t13*(t65*t69 + t72*(t26 + t70) + t74*t77));
    J[1] = T(-t13*(t69*t88 + t72*(t50 + t80) + t77*t90));
    J[2] = T(-t13*(t100*t77 + t69*t98 + t72*(c[0]*t23 - t39 - t40 - t42)));
    J[3] = T(-t13*(t103*t69 + t105*t77 + t72*(t70 + t9)));
    J[4] = T(-t13*(t109*t69 + t111*t77 + t72*(c[0]*t61 + t80 + t91)));
    J[5] = T(-t13*(t114*t69 + t116*t77 + t44*t72));
    J[6] = T(-t38*(t117*((t34) ? (
   0
)
: (
   ((t11) ? (
      t58
   )
   : (
      t57
   ))
)) + t118*((t34) ? (
   0
)
: (
   ((t11) ? (
      t10*t56
   )
   : (
      t73
   ))
)) + t37*(-t46 + t47 + t92)));
    J[7] = T(-t38*(t117*((t34) ? (
   0
)
: (
   ((t11) ? (
      t84
   )
   : (
      -1.0/2.0*t83
   ))
)) + t118*((t34) ? (
   0
)
: (
   ((t11) ? (
      -t10*t83
   )
   : (
      t89
   ))
)) + t37*(t1 + t119 + t3)));
    J[8] = T(-t38*(t117*((t34) ? (
   0
)
: (
   ((t11) ? (
      t95
   )
   : (
      -1.0/2.0*t94
   ))
)) + t118*((t34) ? (
   0
)
: (
   ((t11) ? (
      -t10*t94
   )
   : (
      t99
   ))
)) + t37*(t120 - t14 + t18)));
    J[9] = T(-t38*(t117*((t34) ? (
   0
)
: (
   ((t11) ? (
      t101
   )
   : (
      -1.0/2.0*t20
   ))
)) + t118*((t34) ? (
   0
)
: (
   ((t11) ? (
      -t10*t20
   )
   : (
      t104
   ))
)) + t52));
    J[10] = T(-t38*(t10*t37 + t117*((t34) ? (
   0
)
: (
   ((t11) ? (
      t106
   )
   : (
      -1.0/2.0*t44
   ))
)) + t118*((t34) ? (
   0
)
: (
   ((t11) ? (
      -t10*t44
   )
   : (
      t110
   ))
))));
    J[11] = T(t38*(-t117*((t34) ? (
   0
)
: (
   t113
)) - t118*((t34) ? (
   0
)
: (
   ((t11) ? (
      -t10*t51
   )
   : (
      t115
   ))
)) + t20*t32*t36));
    J[12] = T(-t53*(t122*t65 + t124*t74 + t72*(t123 + t39 + t85)));
    J[13] = T(-t53*(t122*t88 + t124*t90 + t72*(-t15 - t19 - t59)));
    J[14] = T(-t53*(t100*t124 + t122*t98 + t72*(t119 + t24 + t4)));
    J[15] = T(-t53*(t103*t122 + t105*t124 + t72*(t123 + t42 + t81)));
    J[16] = T(-t53*(t109*t122 + t111*t124 + t72*(t120 + t62 + t66)));
    J[17] = T(-t53*(t10*t72 + t114*t122 + t116*t124));
  }
};

// SFG_FACTOR_BARRON_VEC5: Barron-whitened x - y, alpha from mu
// Generated by symforce_gb300.codegen from a sympy residual: 5 residual rows, tangent
// dimension 5; residual in FP64, Jacobian (row-major) in T.
struct GenBarronVec5 {
  static constexpr int NK = 1, NC = 7, RD = 5, TD = 5, MK = 0;
  static constexpr int kTangent[NK] = {5};
  static constexpr int kStorage[NK] = {5};
  static constexpr SFG_HD int KT(int k) { return (k == 0 ? 5 : 0); }
  static constexpr SFG_HD int KS(int k) { return (k == 0 ? 5 : 0); }
  template <typename T>
  static SFG_HD void Run(const double* const* x, const double* c, double* r, T* J) {
    const double t0 = sqrt(c[6]);
    const double t1 = c[0] - x[0][0];
    const double t2 = 1.0/(-c[5] + c[6] + 1);
    const double t3 = -t2;
    const double t4 = c[6] + ((t2 <= 0) ? (
   t3
)
: (
   t2
));
    const double t5 = 1.0/t4;
    const double t6 = pow(t1, 2)*t5 + 1;
    const double t7 = c[6]*((t2 <= 2) ? (
   1
)
: (
   -1
));
    const double t8 = -1.0/2.0*t2 + (1.0/2.0)*t7 + 1;
    const double t9 = pow(t6, t8);
    const double t10 = 2/(t3 + t7 + 2);
    const double t11 = t10*t4;
    const double t12 = sqrt(c[6] + t11*(t9 - 1));
    const double t13 = c[1] - x[0][1];
    const double t14 = pow(t13, 2)*t5 + 1;
    const double t15 = pow(t14, t8);
    const double t16 = sqrt(c[6] + t11*(t15 - 1));
    const double t17 = c[2] - x[0][2];
    const double t18 = pow(t17, 2)*t5 + 1;
    const double t19 = pow(t18, t8);
    const double t20 = sqrt(c[6] + t11*(t19 - 1));
    const double t21 = c[3] - x[0][3];
    const double t22 = pow(t21, 2)*t5 + 1;
    const double t23 = pow(t22, t8);
    const double t24 = sqrt(c[6] + t11*(t23 - 1));
    const double t25 = c[4] - x[0][4];
    const double t26 = pow(t25, 2)*t5 + 1;
    const double t27 = pow(t26, t8);
    const double t28 = sqrt(c[6] + t11*(t27 - 1));
    const double t29 = t10*t8;
    r[0] = -t0 + t12;
    r[1] = -t0 + t16;
    r[2] = -t0 + t20;
    r[3] = -t0 + t24;
    r[4] = -t0 + t28;
    J[0] = T(-t1*t29*t9/(t12*t6));
    J[1] = T(0);
    J[2] = T(0);
    J[3] = T(0);
    J[4] = T(0);
    J[5] = T(0);
    J[6] = T(-t13*t15*t29/(t14*t16));
    J[7] = T(0);
    J[8] = T(0);
    J[9] = T(0);
    J[10] = T(0);
    J[11] = T(0);
    J[12] = T(-t17*t19*t29/(t18*t20));
    J[13] = T(0);
    J[14] = T(0);
    J[15] = T(0);
    J[16] = T(0);
    J[17] = T(0);
    J[18] = T(-t21*t23*t29/(t22*t24));
    J[19] = T(0);
    J[20] = T(0);
    J[21] = T(0);
    J[22] = T(0);
    J[23] = T(0);
    J[24] = T(-t25*t27*t29/(t26*t28));
  }
};

// SFG_FACTOR_LINEAR_VEC5: J x + b, J 9 x 5
// Generated by symforce_gb300.codegen from a sympy residual: 9 residual rows, tangent
// dimension 5; residual in FP64, Jacobian (row-major) in T.
struct GenLinearVec5 {
  static constexpr int NK = 1, NC = 54, RD = 9, TD = 5, MK = 0;
  static constexpr int kTangent[NK] = {5};
  static constexpr int kStorage[NK] = {5};
  static constexpr SFG_HD int KT(int k) { return (k == 0 ? 5 : 0); }
  static constexpr SFG_HD int KS(int k) { return (k == 0 ? 5 : 0); }
  template <typename T>
  static SFG_HD void Run(const double* const* x, const double* c, double* r, T* J) {
    r[0] = c[0]*x[0][0] + c[1]*x[0][1] + c[2]*x[0][2] + c[3]*x[0][3] + c[45] + c[4]*x[0][4];
    r[1] = c[46] + c[5]*x[0][0] + c[6]*x[0][1] + c[7]*x[0][2] + c[8]*x[0][3] + c[9]*x[0][4];
    r[2] = c[10]*x[0][0] + c[11]*x[0][1] + c[12]*x[0][2] + c[13]*x[0][3] + c[14]*x[0][4] + c[47];
    r[3] = c[15]*x[0][0] + c[16]*x[0][1] + c[17]*x[0][2] + c[18]*x[0][3] + c[19]*x[0][4] + c[48];
    r[4] = c[20]*x[0][0] + c[21]*x[0][1] + c[22]*x[0][2] + c[23]*x[0][3] + c[24]*x[0][4] + c[49];
    r[5] = c[25]*x[0][0] + c[26]*x[0][1] + c[27]*x[0][2] + c[28]*x[0][3] + c[29]*x[0][4] + c[50];
    r[6] = c[30]*x[0][0] + c[31]*x[0][1] + c[32]*x[0][2] + c[33]*x[0][3] + c[34]*x[0][4] + c[51];
    r[7] = c[35]*x[0][0] + c[36]*x[0][1] + c[37]*x[0][2] + c[38]*x[0][3] + c[39]*x[0][4] + c[52];
    r[8] = c[40]*x[0][0] + c[41]*x[0][1] + c[42]*x[0][2] + c[43]*x[0][3] + c[44]*x[0][4] + c[53];
    J[0] = T(c[0]);
    J[1] = T(c[1]);
    J[2] = T(c[2]);
    J[3] = T(c[3]);
    J[4] = T(c[4]);
    J[5] = T(c[5]);
    J[6] = T(c[6]);
    J[7] = T(c[7]);
    J[8] = T(c[8]);
    J[9] = T(c[9]);
    J[10] = T(c[10]);
    J[11] = T(c[11]);
    J[12] = T(c[12]);
    J[13] = T(c[13]);
    J[14] = T(c[14]);
    J[15] = T(c[15]);
    J[16] = T(c[16]);
    J[17] = T(c[17]);
    J[18] = T(c[18]);
    J[19] = T(c[19]);
    J[20] = T(c[20]);
    J[21] = T(c[21]);
    J[22] = T(c[22]);
    J[23] = T(c[23]);
    J[24] = T(c[24]);
    J[25] = T(c[25]);
    J[26] = T(c[26]);
    J[27] = T(c[27]);
    J[28] = T(c[28]);
    J[29] = T(c[29]);
    J[30] = T(c[30]);
    J[31] = T(c[31]);
    J[32] = T(c[32]);
    J[33] = T(c[33]);
    J[34] = T(c[34]);
    J[35] = T(c[35]);
    J[36] = T(c[36]);
    J[37] = T(c[37]);
    J[38] = T(c[38]);
    J[39] = T(c[39]);
    J[40] = T(c[40]);
    J[41] = T(c[41]);
    J[42] = T(c[42]);
    J[43] = T(c[43]);
    J[44] = T(c[44]);
  }
};

// SFG_FACTOR_LINEAR_SCALAR2: J [x, y] + b, J 2 x 2
// Generated by symforce_gb300.codegen from a sympy residual: 2 residual rows, tangent
// dimension 2; residual in FP64, Jacobian (row-major) in T.
struct GenLinearScalar2 {
  static constexpr int NK = 2, NC = 6, RD = 2, TD = 2, MK = 0;
  static constexpr int kTangent[NK] = {1, 1};
  static constexpr int kStorage[NK] = {1, 1};
  static constexpr SFG_HD int KT(int k) { return (k == 0 ? 1 : (k == 1 ? 1 : 0)); }
  static constexpr SFG_HD int KS(int k) { return (k == 0 ? 1 : (k == 1 ? 1 : 0)); }
  template <typename T>
  static SFG_HD void Run(const double* const* x, const double* c, double* r, T* J) {
    r[0] = c[0]*x[0][0] + c[1]*x[1][0] + c[4];
    r[1] = c[2]*x[0][0] + c[3]*x[1][0] + c[5];
    J[0] = T(c[0]);
    J[1] = T(c[1]);
    J[2] = T(c[2]);
    J[3] = T(c[3]);
  }
};

}  // namespace sfg

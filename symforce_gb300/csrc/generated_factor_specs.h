// Generated by `python -m symforce_gb300.codegen --write` from the sympy residuals in
// symforce_gb300/factor_defs.py; do not edit by hand.
#pragma once

// X(kind, num_keys, num_consts, residual_dim, key type 0, key type 1, key type 2, struct)
#define SFG_GENERATED_FACTORS(X) \
  X(SFG_FACTOR_PRIOR_ROT3, 1, 8, 3, 6, 0, 0, GenPriorRot3) \
  X(SFG_FACTOR_BETWEEN_ROT3, 2, 8, 3, 6, 6, 0, GenBetweenRot3) \
  X(SFG_FACTOR_BARRON_VEC5, 1, 7, 5, 8, 0, 0, GenBarronVec5) \
  X(SFG_FACTOR_LINEAR_VEC5, 1, 54, 9, 8, 0, 0, GenLinearVec5) \
  X(SFG_FACTOR_LINEAR_SCALAR2, 2, 6, 2, 1, 1, 0, GenLinearScalar2)

"""GB300-native MTCalc solve stage: COCR with the folded preconditioner on
sm_103a, behind a C ABI that mirrors the reference's PCOCR_2x2_Folded."""

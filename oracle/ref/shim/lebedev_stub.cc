// Stand-in for libs/libTriInt/LebedevRules.cc, which the reference tree lacks
// (listed at libs/libTriInt/Makefile.am:6).  Only the displaced-surface-integral
// power method (DSIPFT.cc:301) asks for a Lebedev rule; the oracle never uses
// that method, so the stub reports "no rule".
double *GetLebedevRule(int NumPts) { (void)NumPts; return 0; }

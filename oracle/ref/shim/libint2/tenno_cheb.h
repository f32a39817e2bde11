/* Stand-in for the missing geminal Chebyshev table (out-of-scope operators).
 * Included inside class TennoGmEval; never instantiated.  Test-only shim. */
static constexpr int interpolation_order = 1;
static constexpr int cheb_table_nintervals = 1;
static constexpr int cheb_table_mmax = 0;
static constexpr int cheb_table_tmaxlog2 = 1;
static constexpr int cheb_table_tminlog2 = 0;
static constexpr int cheb_table_umaxlog10 = 1;
static constexpr int cheb_table_uminlog10 = 0;
static constexpr double cheb_table[1][8] = {{0, 0, 0, 0, 0, 0, 0, 0}};

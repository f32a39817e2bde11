/* Stand-in for the missing Chebyshev table blob (absent from the reference
 * tree).  Included inside class FmEval_Chebyshev7; the shimmed reference
 * build never instantiates that class.  Test-only shim. */
static constexpr int interpolation_order = 7;
static constexpr int cheb_table_nintervals = 1;
static constexpr int cheb_table_mmax = 0;
static constexpr double cheb_table_tmax = 1.0;
static constexpr double cheb_table_delta = 1.0;
static constexpr double cheb_table[1][8] = {{0, 0, 0, 0, 0, 0, 0, 0}};

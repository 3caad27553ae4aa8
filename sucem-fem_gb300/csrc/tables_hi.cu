// Reference tables of the N1curl element of orders 3 and 4 (generated by
// gen_tables.py into n1curl_tables_hi.h), in a translation unit of their
// own so their large initialisers compile beside the kernels.
#include "n1curl_tables_hi.h"

namespace sucem {

// which: 0 = KC[6][n][n], 1 = KM[6][n][n], 2 = KT[4][3][n][n]; the
// element dimension n is 45 (order 3) or 84 (order 4).  Null otherwise.
const double* n1curl_table_hi(int order, int which) {
  if (order == 3) return which == 0 ? &KC3[0][0][0] : which == 1 ? &KM3[0][0][0] : &KT3[0][0][0][0];
  if (order == 4) return which == 0 ? &KC4[0][0][0] : which == 1 ? &KM4[0][0][0] : &KT4[0][0][0][0];
  return nullptr;
}

}  // namespace sucem

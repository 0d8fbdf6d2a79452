/* Case-insensitive-filesystem alias used by BuildMatrix/T_Brick.h. */
#include "vec_prep_data.h"

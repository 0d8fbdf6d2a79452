/* Case-insensitive-filesystem alias: some reference sources include
 * "StdAfx.h" while the file on disk is "stdafx.h". */
#include "stdafx.h"

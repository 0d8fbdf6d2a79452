/* Empty stand-in for the MSVC <tchar.h> header, which the reference's
 * precompiled-header files include but never use. */
#pragma once

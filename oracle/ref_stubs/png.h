/* Empty stand-in for libpng's header.  The reference includes <png.h> from
 * parameters.h:21 but calls nothing from it; libpng is not installed here. */
#ifndef RAPTOR_ORACLE_PNG_STUB_H
#define RAPTOR_ORACLE_PNG_STUB_H
#endif

/* Internal helpers shared by the translation units of libprml_gb300.so. */
#ifndef PRML_INTERNAL_H
#define PRML_INTERNAL_H

#include <string>

#include "pararealml_gb300.h"

/* Records `msg` as the calling thread's last error and returns `code`. */
int prml_set_error(int code, const std::string& msg);

#endif

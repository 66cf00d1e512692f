// genie/genie.h -- the C++ interface of the GB300-native GENIE search, a
// drop-in for the reference's <genie/genie.h> (src/genie/genie.h).  It is a
// thin layer over the C ABI of <genie_gb300.h>.
#ifndef GENIE_GENIE_H_
#define GENIE_GENIE_H_

#include <genie/exception/exception.h>
#include <genie/interface/config.h>
#include <genie/interface/execution_policy.h>
#include <genie/interface/io.h>
#include <genie/interface/search.h>
#include <genie/interface/types.h>

#endif

/*
 * sep.h - umbrella header of the sep C API (GB300 implementation).
 * Programs include this one header, as with the reference's include/sep.h:20-31.
 */
#ifndef SEP_GB300_SEP_H
#define SEP_GB300_SEP_H

#include "sepstrct.h"
#include "sepinit.h"
#include "sepprfrc.h"
#include "sepintgr.h"
#include "sepmol.h"
#include "sepmisc.h"
#include "sepret.h"
#include "sepcoulomb.h"
#include "sepsampler.h"
#include "separray.h"
#include "sepgpu.h"

#endif

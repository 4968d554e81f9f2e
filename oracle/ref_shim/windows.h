/* Test infrastructure for the oracle: an empty stand-in so that the reference's
 * IniParser.h (which includes <windows.h> but uses nothing from it) builds on Linux. */
#pragma once

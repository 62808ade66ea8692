/* empty stand-in: the emulation harness performs sorts and scans itself */
#pragma once

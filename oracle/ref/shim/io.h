/* Linux stand-in for the Windows <io.h> header (oracle build only). */
#pragma once
#include <unistd.h>

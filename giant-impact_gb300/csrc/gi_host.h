// gi_host.h -- internal prototypes shared by the host-side translation units.
#pragma once

/* Host-emulation shim (oracle/ref_host): nothing to declare. */
#pragma once

/* Shim: empty stand-in for metal-cpp's Foundation header. Test only. */
#pragma once

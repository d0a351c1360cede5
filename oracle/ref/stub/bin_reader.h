// Empty stand-in for a header that the reference's src/main.cpp:8 includes
// but that the reference does not ship. Nothing from it is used on the path.
#pragma once

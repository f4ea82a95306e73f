// Include-only stand-in: the reference includes this header but the
// compiled hot-path sources use nothing from it.
#pragma once

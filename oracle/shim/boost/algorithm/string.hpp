// Include-only stand-in: the reference names namespace boost here but the
// compiled hot-path sources use nothing from it.
#pragma once
namespace boost {}

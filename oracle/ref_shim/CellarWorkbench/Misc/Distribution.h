// Stand-in for a CellarWorkbench header the reference includes but whose
// contents the compiled checker does not use.  TEST INFRASTRUCTURE ONLY.
#pragma once

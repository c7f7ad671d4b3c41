// Test infrastructure: forwards to the glm API subset used to compile the reference headless.
#include "../glm.hpp"

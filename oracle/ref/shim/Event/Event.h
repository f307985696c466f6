// Stand-in for the engine's Event/Event.h (reference-build recipe, test infrastructure).
#pragma once
class Event {};

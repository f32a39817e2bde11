/* Empty stand-in: the full C++ API header pulls in Engine (needs the generated library). */

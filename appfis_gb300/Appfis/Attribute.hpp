/*
 * Attribute.hpp — run attributes (same fields and defaults as the reference,
 * Appfis/Attribute.hpp:16-24): ghost layers, host threads, periodic boundaries, overlap.
 * `threads` and `overlap` are accepted for source compatibility; the GPU engine ignores them.
 */
#ifndef APPFIS_GB_ATTRIBUTE_HPP
#define APPFIS_GB_ATTRIBUTE_HPP

namespace APPFIS
{

	struct Attribute {
		Attribute() : ghostLayer(1), threads(1), periodic(false), overlap(false) {}
		int ghostLayer;
		int threads;
		bool periodic;
		bool overlap;
	};

	static Attribute ATTRIBUTE;

}

#endif

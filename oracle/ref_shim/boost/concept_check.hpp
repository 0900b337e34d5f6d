// Stand-in for Boost.ConceptCheck (dax/cont/ArrayHandle.h:27): concept
// assertions become no-ops. Test infrastructure only.
#pragma once
#define BOOST_CONCEPT_ASSERT(x) typedef int boost_concept_assert_unused_

"""GB300-native (sm_103a) quadtree spatial join with cuSpatial's API.

Functions mirror cuspatial.quadtree_on_points, polygon_bounding_boxes,
linestring_bounding_boxes, join_quadtree_and_bounding_boxes,
quadtree_point_in_polygon and quadtree_point_to_nearest_linestring, the
unindexed point_in_polygon / pairwise_point_in_polygon, contains_properly and
the pairwise point-linestring distance and nearest points;
they run hand-written CUDA kernels in libcuspatial_gb300.so through its C ABI.
"""

from .api import (HostRowsTooFew, join_quadtree_and_bounding_boxes, last_edge_free_pairs,
                  last_nearest_stats,
                  last_refined_count,
                  linestring_bounding_boxes, pairwise_point_in_polygon,
                  pairwise_point_linestring_distance, pairwise_point_linestring_nearest_points,
                  point_in_polygon, point_in_polygon_bitmask, point_in_polygon_join_host,
                  points_in_quadtree_order,
                  polygon_bounding_boxes, quadtree_on_points, quadtree_on_points_host, quadtree_on_points_ordered,
                  quadtree_point_in_polygon,
                  quadtree_point_in_polygon_host, quadtree_point_to_nearest_linestring)
from .contains import contains_properly, polygons_contains_properly
from .geoseries import GeoSeries, Table

__all__ = [
    "GeoSeries",
    "HostRowsTooFew",
    "Table",
    "contains_properly",
    "join_quadtree_and_bounding_boxes",
    "last_edge_free_pairs",
    "last_nearest_stats",
    "last_refined_count",
    "linestring_bounding_boxes",
    "pairwise_point_in_polygon",
    "pairwise_point_linestring_distance",
    "pairwise_point_linestring_nearest_points",
    "point_in_polygon",
    "point_in_polygon_bitmask",
    "point_in_polygon_join_host",
    "points_in_quadtree_order",
    "polygon_bounding_boxes",
    "polygons_contains_properly",
    "quadtree_on_points",
    "quadtree_on_points_host",
    "quadtree_on_points_ordered",
    "quadtree_point_in_polygon",
    "quadtree_point_in_polygon_host",
    "quadtree_point_to_nearest_linestring",
]
